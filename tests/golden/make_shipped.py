"""Fixture of the reference's one shipped configuration and its data files.

The reference ships one real run set-up: params.i (a 256x1x300 box, 400 Mm,
2 s steps, magnetic, displacement form, PML 10 at the bottom), the Instruction
files Spectral / Adjoint ('2D' selects options 17 and 18), the background
table `polytrope` (300 rows: r/Rsun, c, rho, p, g, Gamma1 in cgs) and, under
data/, the ridge-filter settings params.0 / params.1 (mindist, maxdist,
window), the band corners filter.params.0 / .1 (mHz) and the source position
master.pixels (Mm).  This script reads them where the reference is mounted,
through this package's own parsers (SparcParams.from_params_i, .instruction,
background.read_polytrope), and writes the values to shipped_inputs.npz, so
that tests which run where the reference is absent still use the reference's
own inputs.

Run:  python tests/golden/make_shipped.py /root/reference
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "shipped_inputs.npz")


def read_shipped(ref: str) -> dict:
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    from sparc_gb300.background import read_polytrope
    from sparc_gb300.params import SparcParams
    p = SparcParams.from_params_i(open(os.path.join(ref, "params.i")).read())
    pf = p.instruction(open(os.path.join(ref, "Spectral")).read())
    pa = p.instruction(open(os.path.join(ref, "Adjoint")).read())
    fields = ("nx", "ny", "nz", "xlength", "ylength", "timestep", "npmlbot", "npmltop", "option",
              "damp_waves", "excitdep", "obsheight", "cadforcing", "outputcad", "nupeak", "nuwidth", "solartime")
    data = os.path.join(ref, "data")

    def nums(name):
        return [float(v) for v in open(os.path.join(data, name)).read().split()]

    return {
        "params": {k: getattr(pf, k) for k in fields},
        "adjoint_option": pa.option,
        "polytrope": read_polytrope(os.path.join(ref, "polytrope"), pf.nz),
        "ridges": {0: nums("params.0"), 1: nums("params.1")},
        "bands": {0: nums("filter.params.0"), 1: nums("filter.params.1")},
        "master_pixels": nums("master.pixels"),
    }


def write(d: dict, path: str = OUT) -> None:
    np.savez_compressed(path, params=json.dumps(d["params"]), adjoint_option=d["adjoint_option"],
                        polytrope=d["polytrope"],
                        ridges=np.array([d["ridges"][0], d["ridges"][1]]),
                        bands=np.array([d["bands"][0], d["bands"][1]]),
                        master_pixels=np.array(d["master_pixels"]))


def load(path: str = OUT) -> dict:
    """The shipped configuration: SparcParams of the forward (Spectral) run,
    the adjoint option, the polytrope table, ridges {set: (mindist, maxdist,
    window)}, bands {set: (left, right)} and the source x of master.pixels."""
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    from sparc_gb300.params import SparcParams
    z = np.load(path)
    p = SparcParams(**json.loads(str(z["params"])))
    return {"params": p, "adjoint_option": int(z["adjoint_option"]), "polytrope": z["polytrope"],
            "ridges": {i: tuple(r) for i, r in enumerate(z["ridges"])},
            "bands": {i: tuple(b) for i, b in enumerate(z["bands"])},
            "x00": float(z["master_pixels"][0])}


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    write(read_shipped(ref))
    print(OUT)
