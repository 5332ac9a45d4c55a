"""HBM byte model of the time step (used by bench.py for the roofline line).

Units: one *field access* = one read or write of a whole spectral field of
one source: M * nz complex values, M = ny * (nx/2 + 1), i.e. (nx/2+1)/nx of
the bytes of the physical field (4.03 B per grid point in FP32, 8.06 B in
FP64 at nx = 256).

Algorithmic (compulsory) accesses of the spectral-column schedule:
  RK stage 1 (temp = a):            read a (6 fields)           + write scr (6) = 12
  RK stages 2-5 (temp = a+beta scr): read a (6) + read scr (6)  + write scr (6) = 18
  update + filters:                  read a (6) + read scr (6)  + write a (6)   = 18
  per step: 12 + 4*18 + 18 = 102 accesses.
PML auxiliaries add 2 fields on nzpml planes per pass (counted exactly below).

Implemented accesses of the current stage kernel (four z sweeps with the
tridiagonal intermediates y, p', rho' round-tripping through global memory):
  stage 2-5: S1 2r+1w, S2 11r+6w, S3 1r+1w, S4 4r+2w = 28;  stage 1: 21.
The difference (10 accesses per stage) is the traffic that an on-chip schedule
removes.

The fused FP32 step (fused.cu) keeps a pencil's state on chip for the whole
step: per step it reads a (6 fields) and writes a (6 fields), plus the PML
planes (2 fields on nzpml planes, read + write) and one source plane per
source; the stage right-hand side scr (6 fields) is written only on steps whose
outputs need it.  Its algorithmic and implemented counts coincide: 12 field
accesses per step, against 102 for the per-stage schedule.
"""
from __future__ import annotations

STAGE1_ALG = 12
STAGE_ALG = 18
UPDATE_ALG = 18
STAGE1_IMPL = 21
STAGE_IMPL = 28
UPDATE_IMPL = 18


def complex_bytes(precision: str) -> int:
    return 16 if precision == "f64" else 8


def field_bytes(p, nsrc: int | None = None) -> int:
    """Bytes of one spectral field for all sources of a context."""
    s = p.nsrc if nsrc is None else nsrc
    return (p.nx // 2 + 1) * p.ny * p.nz * complex_bytes(p.precision) * s


def pml_field_bytes(p, nsrc: int | None = None) -> int:
    s = p.nsrc if nsrc is None else nsrc
    return (p.nx // 2 + 1) * p.ny * p.nzpml * complex_bytes(p.precision) * s


def stage_alg_bytes(p, rk: int) -> int:
    """Algorithmic bytes of one launch of RK stage rk (1..5) for all sources."""
    f = field_bytes(p)
    pf = pml_field_bytes(p)
    if rk == 1:
        return STAGE1_ALG * f + (2 + 2) * pf        # read psi, write scrpml
    return STAGE_ALG * f + (4 + 2) * pf             # read psi + scrpml, write scrpml


def stage_impl_bytes(p, rk: int) -> int:
    f = field_bytes(p)
    pf = pml_field_bytes(p)
    return (STAGE1_IMPL if rk == 1 else STAGE_IMPL) * f + (4 if rk == 1 else 6) * pf


def update_alg_bytes(p) -> int:
    return UPDATE_ALG * field_bytes(p) + 6 * pml_field_bytes(p)


def step_alg_bytes(p) -> int:
    return sum(stage_alg_bytes(p, rk) for rk in range(1, 6)) + update_alg_bytes(p)


def step_impl_bytes(p) -> int:
    return sum(stage_impl_bytes(p, rk) for rk in range(1, 6)) + update_alg_bytes(p)


def alg_bytes_per_point_step(p) -> float:
    return step_alg_bytes(p) / (p.points * p.nsrc)


#: Compulsory field accesses per grid-point-step of the minimal per-stage
#: schedule of the reference's physical-space formulation (displacement form,
#: option 4, displacement.f90:482-658 within step.f90:43-128): per RK stage two
#: horizontal passes (H1: read xi_x, xi_y from a and scr, write the horizontal
#: divergence = 5; H2: read p', v_x, v_y from a and scr, write scr v_x, v_y,
#: xi_x, xi_y = 9), the v_z damping pass (3) and two z-pencil passes (Z1: read
#: xi_z from a and scr and the divergence, write p', rho' = 5; Z2: read p',
#: rho', damped v_z and v_z from a and scr, write scr v_z, xi_z = 7), 29 per
#: stage; the update with the z filter (read a and scr, write a: 18) and the
#: horizontal filter every 30 steps (10 / 30).  5 * 29 + 18 + 1/3 = 163.33.
#: This is the per-unit figure the roofline's `achieved` uses: the work of one
#: grid-point-step is credited with the bytes that the minimal per-stage
#: schedule must move for it, whatever the kernel itself moves.
REFERENCE_SCHEDULE_ACCESSES = 5 * 29 + 18 + 10.0 / 30.0


def reference_schedule_bytes_per_point_step(precision: str) -> float:
    """653.3 B (FP32) / 1306.7 B (FP64) per grid-point-step."""
    return REFERENCE_SCHEDULE_ACCESSES * (4 if precision == "f32" else 8)


#: Linearised MHD, displacement form (option 10, the flux tube): the
#: compulsory field accesses per grid-point-step of the minimal schedule.
#: Per stage: the quiet form's 29, the three induction intermediates b
#: (written, then read by the curl pass), their three derivative passes and
#: the Lorentz terms, and 14 three-dimensional background fields (B0, curl
#: B0, the horizontal gradients of p0 and rho0, and the ones the quiet form
#: holds as z columns); about 81 accesses.  Five stages and the update with
#: the z filter of six fields (18) make 423 per point-step: 1.69 kB in FP32,
#: 3.38 kB in FP64.  This is the per-unit figure of the flux-tube roofline.
MHD_SCHEDULE_ACCESSES = 5 * 81 + 18


def mhd_schedule_bytes_per_point_step(precision: str) -> float:
    """1692 B (FP32) / 3384 B (FP64) per grid-point-step of option 10."""
    return MHD_SCHEDULE_ACCESSES * (4 if precision == "f32" else 8)


FUSED_STEP = 12


def fused_step_alg_bytes(p, write_scr: bool = False) -> int:
    """Bytes of one fused-step launch (all sources)."""
    f = field_bytes(p)
    pf = pml_field_bytes(p)
    plane = (p.nx // 2 + 1) * p.ny * complex_bytes(p.precision) * p.nsrc
    return (FUSED_STEP + (6 if write_scr else 0)) * f + 4 * pf + plane


#: DRAM traffic (read + write) of one fused-step launch per source:
#: dram__bytes_read.sum + dram__bytes_write.sum of one ncu capture of a
#: single-source forward step (no scr written) at 256x256x300 FP32.  Traffic
#: grows in proportion to the number of sources, so a batched launch is
#: credited with this figure times nsrc; it is a scaled constant, not a
#: measurement of the run that reports it.
MEASURED_FUSED_TRAFFIC_PER_SOURCE = {(256, 256, 300, "f32"): 920.0e6}

#: Warp instructions executed by one fused-step launch per source
#: (smsp__inst_executed.sum of the same ncu capture), for the issue-side
#: roofline: a launch of nsrc sources issues this many times nsrc.
MEASURED_FUSED_WARP_INST_PER_SOURCE = {(256, 256, 300, "f32"): 424.3e6}


def fused_traffic_per_launch(p):
    v = MEASURED_FUSED_TRAFFIC_PER_SOURCE.get((p.nx, p.ny, p.nz, p.precision))
    return None if v is None else v * p.nsrc


def fused_warp_inst_per_launch(p):
    v = MEASURED_FUSED_WARP_INST_PER_SOURCE.get((p.nx, p.ny, p.nz, p.precision))
    return None if v is None else v * p.nsrc
