"""ctypes binding of libsparc_gpu.so (the C ABI of include/sparc_gpu.h).

This is the Python side of the drop-in boundary: the reference's Python
scripts (full.py, linesearch.py, data_forward.py) shell out to the Fortran
executable; here they would import this module instead.  The library is the
only compute path -- there is no CPU fallback, and loading fails loudly when
the shared object is missing or cannot be loaded.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libsparc_gpu.so")

SPARC_OK = 0
SPARC_EINVAL = -1
SPARC_ENOMEM = -2
SPARC_ECUDA = -3
SPARC_ETIMEDOUT = -4
SPARC_ENAN = -5
SPARC_ESTATE = -6
SPARC_EIO = -7
SPARC_FP64 = 0
SPARC_FP32 = 1
SRC_NONE, SRC_SERIES, SRC_LAGRANGE = 0, 1, 2
ZTAB_ROWS, PTAB_ROWS = 25, 4      # SPARC_ZTAB_ROWS / SPARC_PTAB_ROWS of the header

#: every function the header declares (checked by the CPU test suite)
EXPORTS = [
    "sparc_gpu_create", "sparc_gpu_destroy", "sparc_gpu_errstr", "sparc_gpu_last_error",
    "sparc_gpu_abi_version", "sparc_gpu_set_background", "sparc_gpu_set_source",
    "sparc_gpu_step", "sparc_gpu_stage", "sparc_gpu_get_time", "sparc_gpu_set_time", "sparc_gpu_get_field",
    "sparc_gpu_set_state", "sparc_gpu_get_state", "sparc_gpu_record_surface",
    "sparc_gpu_get_records", "sparc_gpu_checkpoint", "sparc_gpu_restore",
    "sparc_gpu_save_device", "sparc_gpu_load_device", "sparc_gpu_slot_reset", "sparc_gpu_slot_time",
    "sparc_gpu_set_active", "sparc_gpu_set_rhs_output", "sparc_gpu_set_stream_priority", "sparc_gpu_query",
    "sparc_gpu_snapshot", "sparc_gpu_kernel_accumulate", "sparc_gpu_kernel_reset",
    "sparc_gpu_kernels", "sparc_gpu_ddx", "sparc_gpu_ddy", "sparc_gpu_ddz", "sparc_gpu_damp",
    "sparc_gpu_stream", "sparc_gpu_launch_count", "sparc_gpu_device_bytes", "sparc_gpu_info",
    "sparc_gpu_sync", "sparc_gpu_spec_to_phys_noalloc", "sparc_gpu_autotune", "sparc_gpu_set_mhd_background",
    "sparc_gpu_set_mhd2d_background", "sparc_gpu_kernels_b", "sparc_gpu_adjoint_source",
    "sparc_gpu_adjoint_source_host", "sparc_gpu_misfit_all", "sparc_gpu_gradient", "sparc_gpu_update_models",
    "sparc_gpu_kernels_device",
]


class SparcError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"sparc_gpu status {status}: {msg}")
        self.status = status


class CAdjSrcParams(ctypes.Structure):
    """sparc_adjsrc_params (include/sparc_gpu.h)."""
    _fields_ = [
        ("x00", ctypes.c_double), ("t1_min", ctypes.c_double), ("dt_min", ctypes.c_double),
        ("have_ridge", ctypes.c_int * 3), ("ridge", (ctypes.c_double * 3) * 3),
        ("have_band", ctypes.c_int * 2), ("band", (ctypes.c_double * 2) * 2),
        ("linesearch", ctypes.c_int),
    ]


class CParams(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
        ("npmlbot", ctypes.c_int), ("npmltop", ctypes.c_int), ("option", ctypes.c_int),
        ("compute_forward", ctypes.c_int), ("compute_adjoint", ctypes.c_int),
        ("damp_waves", ctypes.c_int), ("src_k", ctypes.c_int), ("precision", ctypes.c_int),
        ("nsrc", ctypes.c_int),
        ("xlength", ctypes.c_double), ("ylength", ctypes.c_double), ("timestep", ctypes.c_double),
        ("excitdep", ctypes.c_double), ("obsheight", ctypes.c_double),
        ("cadforcing", ctypes.c_double), ("outputcad", ctypes.c_double),
        ("nupeak", ctypes.c_double), ("nuwidth", ctypes.c_double), ("solartime", ctypes.c_double),
    ]


_lib = None


def load(path: str | None = None) -> ctypes.CDLL:
    """Load the library; raises if it is absent (no fallback exists)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with sparc_gb300.build.build() "
                           "(there is no CPU fallback)")
    L = ctypes.CDLL(path)
    P = ctypes.c_void_p
    D = ctypes.POINTER(ctypes.c_double)
    I = ctypes.c_int
    sig = {
        "sparc_gpu_create": ([ctypes.POINTER(CParams), ctypes.POINTER(P)], I),
        "sparc_gpu_destroy": ([P], None),
        "sparc_gpu_errstr": ([I], ctypes.c_char_p),
        "sparc_gpu_last_error": ([P], ctypes.c_char_p),
        "sparc_gpu_abi_version": ([], I),
        "sparc_gpu_set_background": ([P, D, D, D, D, D, D], I),
        "sparc_gpu_set_source": ([P, I, I, D, I, D, I], I),
        "sparc_gpu_step": ([P, I], I),
        "sparc_gpu_stage": ([P, I], I),
        "sparc_gpu_get_time": ([P, ctypes.POINTER(I)], I),
        "sparc_gpu_set_time": ([P, I], I),
        "sparc_gpu_get_field": ([P, I, I, I, D], I),
        "sparc_gpu_set_state": ([P, I, D, D], I),
        "sparc_gpu_get_state": ([P, I, D, D], I),
        "sparc_gpu_record_surface": ([P, I, I], I),
        "sparc_gpu_get_records": ([P, I, D, ctypes.POINTER(I)], I),
        "sparc_gpu_checkpoint": ([P, ctypes.c_char_p], I),
        "sparc_gpu_restore": ([P, ctypes.c_char_p], I),
        "sparc_gpu_save_device": ([P, I, I], I),
        "sparc_gpu_load_device": ([P, I], I),
        "sparc_gpu_slot_reset": ([P, I], I),
        "sparc_gpu_slot_time": ([P, I, ctypes.POINTER(I)], I),
        "sparc_gpu_set_active": ([P, I], I),
        "sparc_gpu_set_rhs_output": ([P, I], I),
        "sparc_gpu_set_stream_priority": ([P, I], I),
        "sparc_gpu_query": ([P, ctypes.POINTER(I)], I),
        "sparc_gpu_snapshot": ([P, I, I], I),
        "sparc_gpu_kernel_accumulate": ([P, I, P], I),
        "sparc_gpu_kernel_reset": ([P], I),
        "sparc_gpu_kernels": ([P, I, I, D, D, D], I),
        "sparc_gpu_kernels_device": ([P, I, I, P], I),
        "sparc_gpu_kernels_b": ([P, I, I, D, D, D], I),
        "sparc_gpu_ddx": ([P, D, D], I),
        "sparc_gpu_ddy": ([P, D, D], I),
        "sparc_gpu_ddz": ([P, D, D, I], I),
        "sparc_gpu_damp": ([P, D, D], I),
        "sparc_gpu_stream": ([P], P),
        "sparc_gpu_launch_count": ([P], ctypes.c_longlong),
        "sparc_gpu_device_bytes": ([P], ctypes.c_longlong),
        "sparc_gpu_info": ([P, D, D, D], I),
        "sparc_gpu_sync": ([P, I], I),
        "sparc_gpu_spec_to_phys_noalloc": ([P, P, P, I, P], I),
        "sparc_gpu_autotune": ([P, I, ctypes.POINTER(I), ctypes.POINTER(ctypes.c_float)], I),
        "sparc_gpu_set_mhd_background": ([P, D, D, D, D, D, D], I),
        "sparc_gpu_set_mhd2d_background": ([P, D, D, D, D], I),
        "sparc_gpu_adjoint_source": ([P, I, D, I, ctypes.POINTER(CAdjSrcParams), ctypes.POINTER(I), D, D,
                                      ctypes.POINTER(I)], I),
        "sparc_gpu_adjoint_source_host": ([P, D, D, I, ctypes.POINTER(CAdjSrcParams), ctypes.POINTER(I), D, D,
                                           ctypes.POINTER(I)], I),
        "sparc_gpu_misfit_all": ([P, I, D, D, I, ctypes.POINTER(CAdjSrcParams), ctypes.POINTER(I), D,
                                  ctypes.POINTER(I)], I),
        "sparc_gpu_gradient": ([P, D, D, D, D, D, D], I),
        "sparc_gpu_update_models": ([P, D, D, D, D, D, D, ctypes.c_double, I, D, D, D, D], I),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    if L.sparc_gpu_abi_version() != 1:
        raise RuntimeError("libsparc_gpu ABI version mismatch")
    _lib = L
    return L


def c_params(p) -> CParams:
    return CParams(
        nx=p.nx, ny=p.ny, nz=p.nz, npmlbot=p.npmlbot, npmltop=p.npmltop, option=p.option,
        compute_forward=int(p.compute_forward), compute_adjoint=int(p.compute_adjoint),
        damp_waves=int(p.damp_waves), src_k=int(p.src_k),
        precision=SPARC_FP32 if p.precision == "f32" else SPARC_FP64, nsrc=int(p.nsrc),
        xlength=p.xlength, ylength=p.ylength, timestep=p.timestep, excitdep=p.excitdep,
        obsheight=p.obsheight, cadforcing=p.cadforcing, outputcad=p.outputcad,
        nupeak=p.nupeak, nuwidth=p.nuwidth, solartime=p.solartime)
