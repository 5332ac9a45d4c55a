"""Forward x adjoint sensitivity-kernel workflow for one batch of sources.

The reference runs this as three executions of `sparc` per source
(full.py:62-97): a forward run that writes the surface seismograms and the
partial-state snapshots every 30 s (driver.f90:455-484), an adjoint run driven
by the time-reversed residuals (driver.f90:343-363), and a kernel pass that
pairs forward snapshot k with adjoint snapshot adj_end - k*stepskern
(kernels.f90:197-263) and accumulates K_c, K_rho and the Hessian
(kernels.f90:276-311).

Here the batch stays on the GPU:
  1. forward run 0..maxtime, surface records, device checkpoints at the start
     of every segment of L snapshots;
  2. adjoint source from the residuals at the receivers (host, FP64);
  3. adjoint run 0..maxtime; before it needs forward snapshots of segment g
     (latest segment first), the forward context reloads checkpoint g and
     recomputes that segment into the snapshot store, then the adjoint
     accumulates against it in reversed time order.
Cost: two forward runs and one adjoint run; device memory: G checkpoints and
an L-snapshot store instead of all snapshots.
"""
from __future__ import annotations

import dataclasses

import numpy as np

from . import sources
from .params import SparcParams
from .solver import Solver


def compute_tt(u0: np.ndarray, u: np.ndarray, dt: float) -> float:
    """Travel-time shift by cross-correlation and a parabola through the
    peak, as COMPUTE_TT (driver.f90:921-960)."""
    u0 = np.asarray(u0, dtype=np.float64)
    u = np.asarray(u, dtype=np.float64)
    nt = len(u0)
    lags = np.arange(-nt + 1, nt)
    cc = np.empty(2 * nt - 1)
    for n, i in enumerate(lags):
        if i <= 0:
            l1 = -i                                  # 0-based start of u0
            cc[n] = np.sum(u0[l1:nt] * u[0:nt - l1]) * dt
        else:
            cc[n] = np.sum(u0[0:nt - i] * u[i:nt]) * dt
    loc = int(np.argmax(cc))
    loc = min(max(loc, 1), 2 * nt - 3)
    t = lags[loc - 1:loc + 2] * dt
    mat = np.stack([np.ones(3), t, t * t], axis=1)
    p0, p1, p2 = np.linalg.solve(mat, cc[loc - 1:loc + 2])
    return float(-p1 * 0.5 / p2)


@dataclasses.dataclass
class KernelResult:
    kc: np.ndarray          # (nsrc, nz, ny, nx) or summed (nz, ny, nx)
    krho: np.ndarray
    hessian: np.ndarray
    seismograms: np.ndarray  # (nsrc, nrec, nreceivers) vz at the receivers
    records: np.ndarray      # (nsrc, nrec, ny, nx) surface vz planes


class KernelPipeline:
    """Forward, adjoint and kernel accumulation for p.nsrc sources at once."""

    def __init__(self, p: SparcParams, table: np.ndarray, segment: int = 8):
        self.p = p.replace(compute_forward=True, compute_adjoint=False)
        self.pa = p.replace(compute_forward=False, compute_adjoint=True)
        self.table = np.asarray(table, dtype=np.float64)
        self.L = int(segment)
        self.cad = self.p.steps
        self.maxtime = self.p.maxtime
        self.nt = self.maxtime // self.cad + 1           # snapshots k = 0 .. maxtime/cad

    # ---- 1. forward run ----
    def forward(self, planes, series) -> tuple[Solver, np.ndarray]:
        fwd = Solver(self.p, self.table)
        for s in range(self.p.nsrc):
            fwd.set_source_series(planes[s], series[s] if np.ndim(series) == 2 else series, slot=s)
        G = (self.nt + self.L - 1) // self.L
        fwd.record_surface(self.nt)
        for g in range(G):
            t0 = g * self.L * self.cad
            fwd.step(t0 - fwd.time)
            fwd.save_device(g, G)
        fwd.step(self.maxtime + 1 - fwd.time)
        recs = np.stack([fwd.records(slot=s) for s in range(self.p.nsrc)])
        return fwd, recs

    # ---- 2. adjoint source ----
    def adjoint_planes(self, synth: np.ndarray, obs: np.ndarray, pixels, window=None) -> np.ndarray:
        """synth, obs: (nsrc, nrec, ny, nx) surface records; residual at the
        receiver pixels, time-reversed and windowed -> (nsrc, L, ny, nx)."""
        out = []
        for s in range(self.p.nsrc):
            res = np.stack([synth[s, :, iy, ix] - obs[s, :, iy, ix] for (iy, ix) in pixels])
            out.append(sources.adjoint_planes(self.p, res, pixels, window))
        return np.stack(out)

    # ---- 3. adjoint run with kernel accumulation ----
    def kernels(self, fwd: Solver, adj_planes: np.ndarray, sum_slots: bool = False):
        adj = Solver(self.pa, self.table)
        adj.set_rhs_output(False)              # the adjoint snapshot reads no scr
        for s in range(self.p.nsrc):
            adj.set_source_lagrange(adj_planes[s], slot=s)
        self._accumulate(fwd, adj)
        if sum_slots:
            res = adj.kernels(sum_slots=True)
        else:
            parts = [adj.kernels(slot=s) for s in range(self.p.nsrc)]
            res = tuple(np.stack([q[i] for q in parts]) for i in range(3))
        adj.close()
        return res

    def kernels_device(self, fwd: Solver, adj_planes: np.ndarray, out_ptr: int, stream_sync: bool = True):
        """As kernels(..., sum_slots=True), the sum written into the device
        buffer at out_ptr (3 * N doubles) instead of host arrays."""
        adj = Solver(self.pa, self.table)
        adj.set_rhs_output(False)
        try:
            for s in range(self.p.nsrc):
                adj.set_source_lagrange(adj_planes[s], slot=s)
            self._accumulate(fwd, adj)
            adj.kernels_into(out_ptr, sum_slots=True)
            if stream_sync:
                adj.sync()
        finally:
            adj.close()

    def _accumulate(self, fwd: Solver, adj: Solver):
        """Adjoint run with the kernel accumulation: forward segments
        recomputed from the device checkpoints, latest first."""
        adj.kernel_reset()
        fwd.record_surface(1, enable=False)          # recomputed segments add no records
        G = (self.nt + self.L - 1) // self.L
        for g in range(G - 1, -1, -1):
            k0, k1 = g * self.L, min((g + 1) * self.L, self.nt)
            fwd.load_device(g)
            for k in range(k0, k1):
                fwd.step(k * self.cad + 1 - fwd.time)     # snapshot k: after the step at time k*cad
                fwd.snapshot(k - k0, self.L)
            for k in range(k1 - 1, k0 - 1, -1):
                ia = self.maxtime - k * self.cad
                adj.step(ia + 1 - adj.time)               # adjoint snapshot at time adj_end - k*cad
                adj.kernel_accumulate(fwd, k - k0)

    def run(self, planes, series, obs_records, pixels, window=None, sum_slots=False) -> KernelResult:
        fwd, recs = self.forward(planes, series)
        adjp = self.adjoint_planes(recs, obs_records, pixels, window)
        kc, kr, hs = self.kernels(fwd, adjp, sum_slots)
        fwd.close()
        seis = np.stack([[recs[s, :, iy, ix] for (iy, ix) in pixels] for s in range(self.p.nsrc)])
        return KernelResult(kc, kr, hs, np.swapaxes(seis, 1, 2), recs)


@dataclasses.dataclass
class ShardedResult:
    kernels: object          # torch float64 tensor (3, nz, ny, nx): K_c, K_rho, hessian summed over ALL sources
    sources: list            # global indices of the sources this rank ran
    records: np.ndarray      # (len(sources), nrec, ny, nx) this rank's surface records


def run_sharded(p: SparcParams, table: np.ndarray, planes, series, obs_records, pixels, window=None,
                segment: int = 8, group=None, device=None) -> ShardedResult:
    """The kernel workflow over a global source list on several GPUs (one
    process per GPU): rank r of W runs the sources shard_sources(n, r, W) as
    one batch, writes its kernel sum into a device tensor and the ranks sum
    those with one FP64 all-reduce (grad.py:158-165).  planes, obs_records:
    global lists / arrays indexed by source; series: one series or one per
    source.  Every rank returns the same summed kernels."""
    import torch
    from . import dist as sd
    rank, world = sd.rank_world(group)
    n = len(planes)
    mine = sd.shard_sources(n, rank, world)
    dev = device if device is not None else torch.device("cuda", torch.cuda.current_device())
    ksum = (torch.empty if mine else torch.zeros)((3, p.nz, p.ny, p.nx), dtype=torch.float64, device=dev)
    recs = np.zeros((0, 0, p.ny, p.nx))
    if mine:
        # the library writes ksum on its own stream: nothing of torch's may
        # still be in flight on that memory
        torch.cuda.current_stream(dev).synchronize()
        pl = KernelPipeline(p.replace(nsrc=len(mine)), table, segment)
        ser = [series[i] for i in mine] if np.ndim(series) == 2 else series
        fwd, recs = pl.forward([planes[i] for i in mine], ser)
        try:
            adjp = pl.adjoint_planes(recs, np.asarray(obs_records)[mine], pixels, window)
            pl.kernels_device(fwd, adjp, ksum.data_ptr())
        finally:
            fwd.close()
    sd.reduce_kernels(ksum, group)
    return ShardedResult(ksum, mine, recs)
