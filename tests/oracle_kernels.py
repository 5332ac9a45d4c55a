"""Sensitivity kernels of one source computed by the CPU oracle, in the order
PRODUCE_KERNELS pairs the snapshots (kernels.f90:197-311): every forward
snapshot stored, the adjoint driven by the time-reversed residual at the
receivers, forward snapshot k paired with adjoint snapshot maxtime - k*cad.
Test infrastructure (the checker), small grids only."""
import numpy as np


def kernel_params(**kw):
    from cases import small_params
    base = dict(nx=16, ny=16, nz=32, npmlbot=4, npmltop=4, solartime=0.05, nupeak=0.01, xlength=50e8,
                ylength=50e8)
    base.update(kw)
    return small_params(**base)


def source_kernels(O, p, tab, plane, series, obs, pixels):
    """(3, nz, ny, nx): K_c, K_rho, hessian of one source; obs: (nrec, ny, nx)
    observed surface records."""
    from sparc_gb300 import sources
    cad, mt = p.steps, p.maxtime
    of = O.Oracle(p, tab)
    of.set_source(1, plane[None].copy(), series)
    orad = int(of.info()["o_rad"])
    rsun = of.info()["rsun"]
    fsnap, rec = [], []
    for i in range(mt + 1):
        of.step(1)
        if i % cad == 0:
            a, scr, _ = of.state()
            fsnap.append(np.concatenate([a[0:3], scr[3:6]]))
            rec.append(a[5, orad - 1].copy())
    of.close()
    rec = np.array(rec)
    res = np.stack([rec[:, iy, ix] - obs[:, iy, ix] for (iy, ix) in pixels])
    adjp = sources.adjoint_planes(p, res, pixels)
    oa = O.Oracle(p.replace(compute_forward=False, compute_adjoint=True), tab)
    oa.set_source(2, adjp)
    asnap = []
    for i in range(mt + 1):
        oa.step(1)
        if i % cad == 0:
            asnap.append(oa.state()[0][3:6].copy())
    nt = len(fsnap)
    oa.kernel_reset()
    graw = tab[:, 4] * rsun / 1e12
    for k in range(nt):
        oa.kernel_accumulate(fsnap[k], asnap[nt - 1 - k], graw)
    out = oa.kernel_finish(cad)
    oa.close()
    return out


def global_sources(p, n):
    """n seeded source planes and the zero observations of each."""
    from sparc_gb300 import sources
    rng = np.random.default_rng(11)
    planes = [sources.gaussian_plane(p, 2.0, *rng.uniform(-10, 10, size=2)) for _ in range(n)]
    nrec = p.maxtime // p.steps + 1
    return planes, np.zeros((n, nrec, p.ny, p.nx))
