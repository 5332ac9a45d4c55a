"""A plain stepping run for profilers: one context, one call of N steps.

    python -m sparc_gb300.profile_step --grid 256x256x300 --nsrc 1 --precision f32 --steps 6

Builds the quiet-Sun context of the given grid (the bench's parameters and
polytrope), gives every slot a Gaussian x Ricker forward source, and takes
N steps in one call, so that only the last step writes the stage right-hand
side.  No autotuning: the launch shape is the context's default, or the one
SPARC_FUSED_MODES / the per-stage CTA size selects.  Prints the device time
per step (CUDA events on the context's stream)."""
from __future__ import annotations

import argparse
import json


def main(argv=None) -> int:
    import torch

    from . import sources
    from .background import polytrope_table
    from .params import config_quiet_128, config_quiet_256
    from .solver import Solver

    ap = argparse.ArgumentParser()
    ap.add_argument("--grid", default="256x256x300", help="NXxNYxNZ (128x128x150 or 256x256x300)")
    ap.add_argument("--nsrc", type=int, default=1)
    ap.add_argument("--precision", default="f32", choices=["f32", "f64"])
    ap.add_argument("--steps", type=int, default=6)
    a = ap.parse_args(argv)
    grid = tuple(int(v) for v in a.grid.lower().split("x"))
    base = {(128, 128, 150): config_quiet_128, (256, 256, 300): config_quiet_256}.get(grid)
    if base is None:
        raise SystemExit(f"profile_step: grid {a.grid} is not one of 128x128x150, 256x256x300")
    p = base().replace(precision=a.precision, nsrc=a.nsrc)
    s = Solver(p, polytrope_table(p.nz))
    series = sources.ricker_series(p, a.steps + 64)
    for k in range(a.nsrc):
        s.set_source_series(sources.gaussian_plane(p, 1.0, -40.0 + 80.0 * k / max(a.nsrc, 1), 0.0), series, slot=k)
    st = torch.cuda.ExternalStream(s.stream_ptr)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    s.step(a.steps)
    e1.record(st)
    s.sync(check_finite=True)
    ms = e0.elapsed_time(e1) / a.steps
    print(json.dumps({"grid": list(grid), "nsrc": a.nsrc, "precision": a.precision, "steps": a.steps,
                      "ms_per_step": ms, "launches": s.launches}))
    s.close()
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
