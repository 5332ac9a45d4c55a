"""Serving: continuous batching of solve requests on one GPU.

A request is one forward solve, or a forward solve followed by its adjoint
solve (adjoint source = the time-reversed surface residual at receivers on a
ring around the source), on one of several grid sizes, on the quiet Sun or on
the magnetohydrostatic flux tube (linearised MHD, option 10, the tube on the
box centre, the source anywhere).  The engine keeps, per (grid size, role,
background), pools of batched contexts -- fields resident in HBM, one CUDA
stream each -- and runs an event loop:

  * arrivals join a queue; a queued request is admitted into a free slot of a
    pool of its grid size, or into a new pool if the HBM budget allows one
    (admission by footprint); adjoint phases of finished forward runs are
    admitted first;
  * an admitted slot is reset and starts its own clock at 0 (per-slot clocks
    of the library), so requests join a batch that is already running;
  * every pool with work advances one output interval (steps of 30 s) per
    round; pools run on their own streams, so their work overlaps;
  * a slot whose clock reaches the request's length is finished: its
    seismograms are read back and the slot is free for the next admission.

Results do not depend on the mix: a slot's arithmetic is independent of the
other slots of its batch and of other pools.
"""
from __future__ import annotations

import dataclasses
import time

import numpy as np

from . import sources
from .background import mhs_flux_tube_background, polytrope_table
from .params import OPT_MHD_PML_3D_DISPL, TUBE_EXCITDEP, TUBE_OBSHEIGHT, SparcParams
from .solver import Solver

QUIET, TUBE = "quiet", "tube"


@dataclasses.dataclass
class Request:
    rid: int
    grid: tuple            # (nx, ny, nz)
    kind: str              # "fwd" or "fwd+adj"
    nsteps: int            # time steps per phase (a multiple of the output cadence)
    x0_mm: float
    y0_mm: float
    arrival: float         # seconds after the start of the stream
    admitted: float = -1.0
    finished: float = -1.0
    records: np.ndarray | None = None        # forward surface vz records (nrec, ny, nx)
    adj_records: np.ndarray | None = None    # adjoint surface vz records
    phase: int = 0
    background: str = QUIET                  # QUIET or TUBE

    @property
    def latency(self) -> float:
        return self.finished - self.arrival


def grid_params(grid, precision: str, base: SparcParams | None = None, background: str = QUIET) -> SparcParams:
    """200 Mm periodic box for every grid size; the flux tube runs option 10
    with the PML at the bottom only, receivers and source 200 and 400 km
    below the top (its box ends at the surface)."""
    nx, ny, nz = grid
    b = base or SparcParams()
    length = 200.0e8
    p = b.replace(nx=nx, ny=ny, nz=nz, xlength=length, ylength=length, npmlbot=10, npmltop=10,
                  excitdep=-15000000.0, obsheight=20000000.0, precision=precision)
    if background == TUBE:
        p = p.replace(option=OPT_MHD_PML_3D_DISPL, npmltop=0, obsheight=TUBE_OBSHEIGHT, excitdep=TUBE_EXCITDEP)
    return p


def grid_table(nz: int, background: str = QUIET) -> np.ndarray:
    """The quiet column: -25 .. +1.2 Mm; under the flux tube -25 .. 0 Mm."""
    return polytrope_table(nz) if background == QUIET else polytrope_table(nz, z_bot_mm=-25.0, z_top_mm=0.0)


class Pool:
    """One batched context (one grid size, one role) with `slots` slots."""

    def __init__(self, p: SparcParams, table, role: str, slots: int, max_records: int, background: str = QUIET,
                 tube_cache: dict | None = None, priority: int = 0):
        import torch
        self.role = role
        self.background = background
        self.p = p.replace(nsrc=slots, compute_forward=(role == "fwd"), compute_adjoint=(role == "adj"))
        self.solver = Solver(self.p, table)
        if priority > 0:
            self.solver.set_stream_priority(priority)
        self.stream = torch.cuda.ExternalStream(self.solver.stream_ptr)
        self.inflight: list = []        # events of the queued output intervals, oldest first
        self.done_at: dict = {}         # slot -> event after which its request has all its steps
        if background == TUBE:
            # the magnetohydrostatic tube of this grid, built once (FP64, with
            # this context's FP64 z derivative) and shared by its pools
            key = (self.p.nx, self.p.ny, self.p.nz)
            cache = tube_cache if tube_cache is not None else {}
            if key not in cache:
                cache[key] = mhs_flux_tube_background(self.p, table, self.solver.ddz)[0]
            self.solver.set_mhd_background(*cache[key])
        self.solver.record_surface(max_records)
        self.requests: list = [None] * slots
        self.series = sources.ricker_series(self.p, 8 * max_records * self.p.steps)
        self.max_records = max_records
        self.bytes = self.solver.device_bytes

    @property
    def free(self) -> list:
        return [i for i, r in enumerate(self.requests) if r is None]

    @property
    def busy(self) -> bool:
        return any(r is not None for r in self.requests)

    def admit(self, req: Request, planes=None):
        slot = self.free[0]
        s = self.solver
        if self.role == "fwd":
            s.set_source_series(sources.gaussian_plane(self.p, 1.0, req.x0_mm, req.y0_mm), self.series, slot=slot)
        else:
            # the source buffer is sized by its first use: pad to the maximum length
            padded = np.zeros((self.max_records,) + planes.shape[1:])
            padded[: min(len(planes), self.max_records)] = planes[: self.max_records]
            s.set_source_lagrange(padded, slot=slot)
        s.slot_reset(slot)
        self.requests[slot] = req
        s.set_active(max(i for i, r in enumerate(self.requests) if r is not None) + 1)
        return slot

    def advance(self, nsteps: int) -> bool:
        """Queue nsteps more steps (one step on the flux tube), unless two
        such chunks are still queued: the GPU queues stay short, so the
        streams' priorities decide the order of the pools' work.  A flux-tube
        step is hundreds of separate launches (its per-slot filter schedule
        keeps it out of graphs); queuing one at a time keeps the host from
        blocking on a full launch queue while cheap pools wait.  Returns
        whether steps were queued."""
        import torch
        if not self.busy:
            return False
        while self.inflight and self.inflight[0].query():
            self.inflight.pop(0)
        if len(self.inflight) >= 2:
            return False
        self.solver.step(nsteps if self.background == QUIET else 1)
        ev = torch.cuda.Event()
        ev.record(self.stream)
        self.inflight.append(ev)
        for slot, req in enumerate(self.requests):
            if req is not None and slot not in self.done_at and self.solver.slot_time(slot) >= req.nsteps:
                self.done_at[slot] = ev
        return True

    def collect(self) -> list:
        """Requests whose last step has finished on the GPU (non-blocking),
        with their records up to their own length."""
        done = []
        for slot in sorted(self.done_at):
            if self.done_at[slot].query():
                req = self.requests[slot]
                nrec = req.nsteps // self.p.steps     # the records of its own steps (the slot may have run on)
                done.append((req, self.solver.records(slot=slot)[:nrec]))
                self.requests[slot] = None
                del self.done_at[slot]
        if done and self.busy:
            self.solver.set_active(max(i for i, r in enumerate(self.requests) if r is not None) + 1)
        return done

    def close(self):
        self.solver.close()


#: magnetohydrostatic tube backgrounds per grid (FP64 host arrays, the same
#: for every precision), built on first use and kept for the process
_TUBES: dict = {}


class Engine:
    """Continuous-batching request loop on one GPU."""

    def __init__(self, precision: str = "f32", hbm_budget: float = 200e9, slots: dict | None = None,
                 max_steps: int = 7200, base: SparcParams | None = None):
        self.precision = precision
        self.budget = hbm_budget
        self.slots = slots or {}
        self.max_steps = max_steps
        self.base = base
        self.pools: list[Pool] = []
        self.max_pools_per_key = 2
        self.tables: dict = {}
        self.tubes: dict = _TUBES             # FP64 tube backgrounds, shared by the engines of a process
        self.cad = (base or SparcParams()).steps

    def _table(self, nz, background=QUIET):
        if (nz, background) not in self.tables:
            self.tables[(nz, background)] = grid_table(nz, background)
        return self.tables[(nz, background)]

    def warm(self, backgrounds=(QUIET, TUBE), roles=("fwd", "adj")) -> int:
        """Create one pool per (grid, background, role) of the configured
        slot sizes before requests arrive, cheapest configuration first, as
        far as the HBM budget goes (no pool is released for it).  A server
        does this at start-up, so that no request waits behind a context's
        set-up (allocation, background tables, the FP64 tube equilibrium).
        Returns the number of pools."""
        keys = sorted({(tuple(g), bg) for g in self.slots for bg in backgrounds},
                      key=lambda k: -self._priority(*k))
        for g, bg in keys:
            for role in roles:
                if self._pool_for(g, role, bg, evict=False) is None:
                    return len(self.pools)
        return len(self.pools)

    def _pool_for(self, grid, role, background=QUIET, evict: bool = True) -> Pool | None:
        def mine(pl):
            return pl.role == role and pl.background == background and (pl.p.nx, pl.p.ny, pl.p.nz) == tuple(grid)
        for pl in self.pools:
            if mine(pl) and pl.free:
                return pl
        same = [pl for pl in self.pools if mine(pl)]
        if len(same) >= self.max_pools_per_key:
            return None
        # admission by footprint: a new pool only if it fits the HBM budget,
        # after releasing idle pools (least recently created first)
        p = grid_params(grid, self.precision, self.base, background)
        slots = self.slots.get(tuple(grid), 4)
        field = (p.nx // 2 + 1) * p.ny * p.nz * (8 if self.precision == "f32" else 16)
        est = slots * field * (15 + (self.max_steps // self.cad + 1) / p.nz) + p.points * 12 + 64e6
        if background == TUBE:
            est *= 3.0      # physical state, the MHD work fields and the 3-D background
        if est > self.budget:
            if not evict:
                return None
            raise RuntimeError(f"a {grid} pool needs {est / 1e9:.1f} GB, above the HBM budget")
        while sum(pl.bytes for pl in self.pools) + est > self.budget:
            idle = [pl for pl in self.pools if not pl.busy]
            if not idle or not evict:
                return None
            idle[0].close()
            self.pools.remove(idle[0])
        pl = Pool(p, self._table(p.nz, background), role, slots, self.max_steps // self.cad + 1, background,
                  self.tubes, priority=self._priority(grid, background))
        self.pools.append(pl)
        return pl

    def _priority(self, grid, background) -> int:
        """Stream priority level of a pool: the cheaper a step of its
        configuration (grid points, times about 12 for the flux tube's
        physical-space path), the more urgent, so short requests finish
        first while long ones keep the GPU busy.  0 for the most expensive."""
        def cost(g, bg):
            return g[0] * g[1] * g[2] * (12 if bg == TUBE else 1)
        keys = {(tuple(g), bg) for g in list(self.slots) + [tuple(grid)] for bg in (QUIET, TUBE)}
        ranked = sorted({cost(g, bg) for g, bg in keys}, reverse=True)
        return ranked.index(cost(tuple(grid), background))

    def _adjoint_planes(self, pl: Pool, req: Request):
        pix = sources.receiver_pixels(pl.p, n=8, radius_mm=10.0, x0_mm=req.x0_mm, y0_mm=req.y0_mm)
        res = np.stack([req.records[:, iy, ix] for (iy, ix) in pix])      # residual against zero data
        return sources.adjoint_planes(pl.p, res, pix)

    def run(self, requests: list[Request], time_scale: float = 1.0, max_wall: float = 900.0) -> list[Request]:
        pending = sorted(requests, key=lambda r: r.arrival)
        queue: list[Request] = []
        adj_queue: list[Request] = []
        done: list[Request] = []
        t_start = time.perf_counter()
        while (pending or queue or adj_queue or any(pl.busy for pl in self.pools)):
            now = (time.perf_counter() - t_start) / time_scale
            if (time.perf_counter() - t_start) > max_wall:
                raise RuntimeError("serving stream exceeded its wall-clock limit")
            while pending and pending[0].arrival <= now:
                queue.append(pending.pop(0))
            # admission: adjoint phases first, then new requests (FIFO)
            for q, role in ((adj_queue, "adj"), (queue, "fwd")):
                keep = []
                for req in q:
                    pl = self._pool_for(req.grid, role, req.background)
                    if pl is None:
                        keep.append(req)
                        continue
                    if role == "fwd":
                        req.admitted = now
                        pl.admit(req)
                    else:
                        pl.admit(req, self._adjoint_planes(pl, req))
                q[:] = keep
            if not any(pl.busy for pl in self.pools):
                if pending:
                    time.sleep(max(0.0, min(0.01, (pending[0].arrival - now) * time_scale)))
                    continue
                if queue or adj_queue:
                    # nothing runs, nothing arrives, and the queue cannot be admitted
                    raise RuntimeError("serving: queued requests cannot be admitted within the HBM budget")
                continue
            moved = False
            for pl in self.pools:            # every pool queues one more output interval; streams overlap
                moved |= bool(pl.advance(self.cad))
            finished = 0
            for pl in self.pools:
                for req, recs in pl.collect():
                    finished += 1
                    t = (time.perf_counter() - t_start) / time_scale
                    if pl.role == "fwd":
                        req.records = recs
                        if req.kind == "fwd+adj":
                            req.phase = 1
                            adj_queue.append(req)
                            continue
                    else:
                        req.adj_records = recs
                    req.finished = t
                    done.append(req)
            if not moved and not finished:
                time.sleep(0.0002)           # every pool has two intervals queued
        return done

    def close(self):
        for pl in self.pools:
            pl.close()
        self.pools = []


def poisson_stream(n: int, rate: float = 4.0, seed: int = 0, mix=None, hours=(1.0, 4.0), dt: float = 2.0,
                   cad: int = 15, compress: float = 1.0, p_adj: float = 0.5, p_tube: float = 0.2) -> list[Request]:
    """Seeded request stream: Poisson arrivals, grid mix (60 % 128^2x150,
    30 % 256^2x300, 10 % 512^2x300 by default), random source position,
    forward-only or forward+adjoint, quiet Sun or (a fraction p_tube) the
    flux tube, 1-4 h of solar time divided by `compress` (time steps rounded
    up to the output cadence)."""
    rng = np.random.default_rng(seed)
    mix = mix or [((128, 128, 150), 0.6), ((256, 256, 300), 0.3), ((512, 512, 300), 0.1)]
    grids = [g for g, _ in mix]
    probs = np.array([w for _, w in mix], dtype=float)
    probs /= probs.sum()
    t = 0.0
    out = []
    for i in range(n):
        t += rng.exponential(1.0 / rate)
        g = grids[rng.choice(len(grids), p=probs)]
        hours_i = rng.uniform(*hours)
        steps = int(np.ceil(hours_i * 3600.0 / dt / compress / cad)) * cad
        half = 0.4 * 200.0
        x0, y0 = rng.uniform(-half, half, size=2)
        kind = "fwd+adj" if rng.random() < p_adj else "fwd"
        bgr = TUBE if rng.random() < p_tube else QUIET
        out.append(Request(i, g, kind, steps, float(x0), float(y0), t, background=bgr))
    return out


def latency_stats(done: list[Request]) -> dict:
    """p50/p95/p99 of finish - arrival over all requests, and per background
    (quiet Sun, flux tube) with the admission wait (admitted - arrival)."""
    lat = np.array([r.latency for r in done])
    out = {"n": len(done), "p50_s": float(np.percentile(lat, 50)), "p95_s": float(np.percentile(lat, 95)),
           "p99_s": float(np.percentile(lat, 99)), "mean_s": float(lat.mean())}
    by = {}
    for bg in sorted({r.background for r in done}):
        rs = [r for r in done if r.background == bg]
        lb = np.array([r.latency for r in rs])
        wb = np.array([r.admitted - r.arrival for r in rs])
        by[bg] = {"n": len(rs), "p50_s": float(np.percentile(lb, 50)), "p99_s": float(np.percentile(lb, 99)),
                  "wait_p50_s": float(np.percentile(wb, 50))}
    out["by_background"] = by
    return out


def main(argv=None):
    """python -m sparc_gb300.serving --requests N --compress C --precision f32"""
    import argparse
    import json
    ap = argparse.ArgumentParser()
    ap.add_argument("--requests", type=int, default=48)
    ap.add_argument("--rate", type=float, default=4.0)
    ap.add_argument("--compress", type=float, default=120.0)
    ap.add_argument("--precision", default="f32")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--budget-gb", type=float, default=120.0)
    a = ap.parse_args(argv)
    reqs = poisson_stream(a.requests, rate=a.rate, seed=a.seed, compress=a.compress)
    eng = Engine(precision=a.precision, hbm_budget=a.budget_gb * 1e9,
                 slots={(128, 128, 150): 8, (256, 256, 300): 4, (512, 512, 300): 2},
                 max_steps=max(r.nsteps for r in reqs))
    eng.warm()
    t0 = time.perf_counter()
    done = eng.run(reqs)
    wall = time.perf_counter() - t0
    eng.close()
    st = latency_stats(done)
    pts = sum(r.grid[0] * r.grid[1] * r.grid[2] * r.nsteps * (2 if r.kind == "fwd+adj" else 1) for r in done)
    st.update({"Mpoint_steps_per_s": pts / wall / 1e6, "wall_s": wall})
    print(json.dumps(st))


if __name__ == "__main__":
    main()
