"""Simulation parameters: the drop-in mirror of the reference's ``params.i``
plus its runtime Instruction-file flags.

``params.i`` (params.i:25-150) is a compile-time Fortran include; here the same
quantities live in one dataclass that can also be parsed from a params.i-style
text file (``SparcParams.from_params_i``).  Derived quantities follow
initialize.f90:978-981 (READ_PARAMETERS) and driver.f90:269-283.

Literal kinds: the reference compiles without -r8, so its real literals are
4-byte REALs.  ``r4`` reproduces that rounding for derived constants that the
reference computes from such literals.
"""
from __future__ import annotations

import dataclasses
import math
import re

import numpy as np

#: option codes of step.f90:74-110 that this framework implements
OPT_QUIET_PML_3D = 2           # pml.f90:12 (MP_QUIET_PML_3D), velocity form
OPT_QUIET_PML_3D_DISPL = 4     # displacement.f90:482 (MP_QUIET_PML_3D_DISPL)
OPT_MHD_PML_3D = 8             # pml.f90:80 (MP_MHD_PML_3D), MHD velocity form
OPT_MHD_PML_3D_DISPL = 10      # displacement.f90:663 (MP_MHD_PML_3D_DISPL)
OPT_QUIET_PML_2D_DISPL = 17    # physics2d.f90:948 (MP_QUIET_PML_2D_DISPL)
OPT_MHD_PML_2D_DISPL = 18      # physics2d.f90:724 (MP_MHD_PML_2D_DISPL)
SUPPORTED_OPTIONS = (OPT_QUIET_PML_3D, OPT_QUIET_PML_3D_DISPL, OPT_MHD_PML_3D, OPT_MHD_PML_3D_DISPL,
                     OPT_QUIET_PML_2D_DISPL, OPT_MHD_PML_2D_DISPL)


def r4(x: float) -> float:
    """Round a decimal literal the way a default-kind (REAL*4) Fortran literal is."""
    return float(np.float32(x))


@dataclasses.dataclass
class SparcParams:
    nx: int = 256
    ny: int = 256
    nz: int = 300
    xlength: float = 400.0e8          # cm (params.i:26)
    ylength: float = 400.0e8
    timestep: float = 2.0             # s (params.i:26)
    npmlbot: int = 10                 # params.i:108
    npmltop: int = 0
    option: int = OPT_QUIET_PML_3D_DISPL
    compute_forward: bool = True      # Instruction file 'spectral' (initialize.f90:1013)
    compute_adjoint: bool = False     # Instruction file 'adjoint' (initialize.f90:1034)
    damp_waves: bool = True           # params.i:38
    src_k: int = 0                    # 1-based source plane; 0 -> e_rad (fwd) / o_rad (adj)
    excitdep: float = -50000000.0     # cm (params.i:150)
    obsheight: float = 20000000.0     # cm (params.i:130)
    cadforcing: float = 30.0          # s (params.i:47)
    outputcad: float = 30.0           # s (params.i:136)
    nupeak: float = 0.0017            # Hz (params.i:64)
    nuwidth: float = 0.0055
    solartime: float = 2.0            # h (params.i:129)

    # ---- framework knobs (no reference counterpart) ----
    precision: str = "f64"            # "f64" (plain) or "f32" (bulk FP32, FP64 set-up/accumulation)
    nsrc: int = 1                     # sources batched on the source axis

    def validate(self) -> None:
        if self.option not in SUPPORTED_OPTIONS:
            raise ValueError(f"option {self.option} not supported (have {SUPPORTED_OPTIONS})")
        if self.option in (OPT_QUIET_PML_2D_DISPL, OPT_MHD_PML_2D_DISPL) and self.ny != 1:
            raise ValueError(f"option {self.option} (2-D) needs ny == 1")
        for n in (self.nx,) + ((self.ny,) if self.ny > 1 else ()):
            if n < 4 or (n & (n - 1)) != 0 or n > 1024:
                raise ValueError(f"horizontal size {n} must be a power of two in [4, 1024]")
        if self.nz < 16 or self.nz > 1024:
            raise ValueError("nz must be in [16, 1024]")
        if self.npmlbot < 2 or self.npmlbot > self.nz // 4 or self.npmltop < 0 or self.npmltop > self.nz // 4:
            raise ValueError("PML widths out of range")
        if self.precision not in ("f64", "f32"):
            raise ValueError("precision must be 'f64' or 'f32'")
        if self.nsrc < 1:
            raise ValueError("nsrc must be >= 1")

    # ---- derived (READ_PARAMETERS, initialize.f90:978-981; driver.f90:269-283) ----
    @property
    def cadforcing_step(self) -> int:
        return int(math.floor(r4(self.cadforcing) / r4(self.timestep)))

    @property
    def maxtime(self) -> int:
        ts = r4(self.timestep)
        mt = int(math.floor((r4(self.solartime) * 3600.0 + 2.0 / r4(self.nupeak)) / ts)) + 2
        cs = self.cadforcing_step
        return cs * (mt // cs)

    @property
    def forcing_length(self) -> int:
        return self.maxtime // self.cadforcing_step + 1

    @property
    def steps(self) -> int:
        """Output cadence in time steps (driver.f90:269)."""
        return int(math.floor(r4(self.outputcad) / r4(self.timestep)))

    @property
    def freq_filtering(self) -> int:
        """Horizontal spectral filter cadence (driver.f90:270)."""
        return int(math.floor(60.0 / r4(self.timestep)))

    @property
    def num_steps(self) -> int:
        n = int(math.floor(self.maxtime * r4(self.timestep) / r4(self.cadforcing))) + 2
        return 2 * (n // 2) + 2

    @property
    def nzpml(self) -> int:
        return self.npmlbot + self.npmltop

    @property
    def points(self) -> int:
        return self.nx * self.ny * self.nz

    def replace(self, **kw) -> "SparcParams":
        return dataclasses.replace(self, **kw)

    # ---- params.i text ----
    _KEYS = {
        "nx": int, "ny": int, "nz": int, "xlength": float, "ylength": float,
        "timestep": float, "npmlbot": int, "npmltop": int, "excitdep": float,
        "obsheight": float, "cadforcing": float, "outputcad": float,
        "nupeak": float, "nuwidth": float, "solartime": float,
    }

    @classmethod
    def from_params_i(cls, text: str, **overrides) -> "SparcParams":
        """Parse the ``parameter(name = value, ...)`` statements of a params.i
        file.  Logical switches map as PARSE_OPTIONS (initialize.f90:778-824)
        does for the supported options: USE_PML must be true; without
        MAGNETIC, DISPL selects option 4 (true) or the velocity form, option 2
        (false); MAGNETIC selects option 10 with DISPL, option 8 without; FLOWS
        must be false."""
        vals: dict = {}
        body = re.sub(r"!.*", "", text)
        for m in re.finditer(r"parameter\s*\((.*?)\)\s*$", body, re.I | re.M | re.S):
            for part in re.split(r",(?![^()]*\))", m.group(1)):
                if "=" not in part:
                    continue
                k, v = (s.strip() for s in part.split("=", 1))
                k = k.lower()
                if k in cls._KEYS:
                    vals[k] = _eval_fortran_number(v, vals)
        for m in re.finditer(r"logical[^:\n]*::\s*(\w+)\s*=\s*\.(\w+)\.", body, re.I):
            vals["_" + m.group(1).lower()] = m.group(2).lower() == "true"
        kw = {k: cls._KEYS[k](v) for k, v in vals.items() if not k.startswith("_")}
        if vals.get("_flows"):
            raise ValueError("FLOWS backgrounds are not supported by this framework")
        if "_damp_waves" in vals:
            kw["damp_waves"] = vals["_damp_waves"]
        if vals.get("_displ") is False:
            kw["option"] = OPT_QUIET_PML_3D
        if vals.get("_magnetic"):
            kw["option"] = OPT_MHD_PML_3D if vals.get("_displ") is False else OPT_MHD_PML_3D_DISPL
        kw.update(overrides)
        p = cls(**kw)
        p.validate()
        return p

    def instruction(self, text: str) -> "SparcParams":
        """Apply an Instruction file (initialize.f90:1006-1051): line 1
        'spectral' | 'adjoint', line 2 '2D' or not; 2D turns option 4 into 17
        and option 10 into 18 (PARSE_OPTIONS, initialize.f90:778-824)."""
        lines = [l.strip() for l in text.strip().splitlines()]
        kind = lines[0].lower() if lines else "spectral"
        two_d = len(lines) > 1 and lines[1].upper() == "2D"
        p = self.replace(compute_forward=(kind == "spectral"), compute_adjoint=(kind == "adjoint"))
        if two_d:
            # READ_PARAMETERS turns every 2-D kernel-mode run into option 17
            # or 18 (initialize.f90:315,1081-1084), both displacement forms;
            # with DISPL = .false. the reference has sized the state for the
            # velocity form by then (initialize.f90:310-312)
            if self.option in (OPT_QUIET_PML_3D, OPT_MHD_PML_3D):
                raise ValueError("a 2D instruction selects the displacement forms 17/18; "
                                 "DISPL = .false. has no consistent 2-D run")
            two_d_of = {OPT_QUIET_PML_3D_DISPL: OPT_QUIET_PML_2D_DISPL, OPT_MHD_PML_3D_DISPL: OPT_MHD_PML_2D_DISPL}
            p = p.replace(option=two_d_of.get(self.option, self.option), ny=1)
        return p


def _eval_fortran_number(s: str, known: dict | None = None) -> float:
    """Evaluate a params.i constant expression: numbers (d/e exponents),
    + - * / ** and parentheses, and names defined earlier in the file."""
    expr = s.strip().lower()
    expr = re.sub(r"(?<=[0-9.])d(?=[-+]?[0-9])", "e", expr)
    if not re.fullmatch(r"[0-9a-z_.+\-*/() ]+", expr):
        raise ValueError(f"unsupported params.i expression: {s!r}")
    names = {k: v for k, v in (known or {}).items() if not k.startswith("_")}
    bare = re.sub(r"(\d+\.?\d*|\.\d+)(e[-+]?\d+)?", " ", expr)
    for tok in re.findall(r"[a-z_][a-z_0-9]*", bare):
        if tok not in names:
            raise ValueError(f"unknown name {tok!r} in {s!r}")
    return float(eval(expr, {"__builtins__": {}}, names))


# ---- the workload configurations of the benchmark suite (synthetic inputs) ----
def config_quiet_128() -> SparcParams:
    """128x128x150 quiet Sun, 200 Mm periodic box, PML 10 top + 10 bottom."""
    return SparcParams(nx=128, ny=128, nz=150, xlength=200.0e8, ylength=200.0e8,
                       npmlbot=10, npmltop=10, excitdep=-15000000.0, obsheight=20000000.0,
                       solartime=1.0)


def config_quiet_256() -> SparcParams:
    """256x256x300 quiet Sun, 200 Mm periodic box, PML 10 top + 10 bottom, 4 h."""
    return SparcParams(nx=256, ny=256, nz=300, xlength=200.0e8, ylength=200.0e8,
                       npmlbot=10, npmltop=10, excitdep=-15000000.0, obsheight=20000000.0,
                       solartime=4.0)


def config_flux_tube_256():
    """The flux-tube configuration: option 10 on 256x256x300, 200 Mm
    periodic, PML 10 at the bottom; the box ends at the surface (z = 0),
    where a 2 kG tube can still be in magnetohydrostatic balance with the gas
    pressure (above it the pressure falls by e every ~100 km); receivers
    200 km and the source 400 km below it.  Returns (params, polytrope
    table)."""
    from .background import polytrope_table
    p = config_quiet_256().replace(option=OPT_MHD_PML_3D_DISPL, npmltop=0, obsheight=TUBE_OBSHEIGHT,
                                   excitdep=TUBE_EXCITDEP)
    return p, polytrope_table(p.nz, z_bot_mm=-25.0, z_top_mm=0.0)


#: observation height and source depth of the flux-tube box (cm): its top is
#: z = 0, so the receivers (an adjoint source) and the forward source sit 200
#: and 400 km below it, strictly inside on every grid of 32 levels or more
TUBE_OBSHEIGHT = -2.0e7
TUBE_EXCITDEP = -4.0e7
