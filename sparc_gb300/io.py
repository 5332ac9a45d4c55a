"""The reference's on-disk formats, written and read without CFITSIO.

* ``vz_cc.bin`` -- a Fortran direct-access unformatted file whose record k
  (1-based) holds the surface vz plane of output k as nx*ny REAL*8 values,
  x fastest, in the machine's byte order, no record markers
  (``write_binary_seq_2D``, all_modules.f90:947-1006, opened with
  ``recl = iolength(tempoa(nx,ny))`` at driver.f90:570,637-639);
* FITS primary arrays, BITPIX = -64, NAXIS = 3 with NAXIS1 = nx, NAXIS2 = ny,
  NAXIS3 = planes (``writefits_local`` all_modules.f90:254-293 for vz_cc.fits;
  ``writefits_3D`` all_modules.f90:296-378, which adds the TIME keyword, for
  kernel_c_XX.fits, kernel_rho_XX.fits, hessian_XX.fits, kernels.f90:465,532,539);
  big-endian data in 2880-byte blocks as the FITS standard defines them;
* ``kernel_info`` and ``timeline`` -- list-directed text (driver.f90:307-309,
  346-352, 457): one integer per line, and ``time timeline`` pairs.

Arrays here are numpy arrays in C order [plane][y][x], which is the Fortran
order a(x, y, plane) of the files.
"""
from __future__ import annotations

import os

import numpy as np

FITS_BLOCK = 2880


# ---- vz_cc.bin -----------------------------------------------------------

def write_vz_cc_bin(path: str, planes: np.ndarray, first_record: int = 1) -> None:
    """Write planes (nrec, ny, nx) as records first_record, first_record+1, ...
    of a direct-access file, creating or extending it (records before
    first_record that do not exist yet read as zeros)."""
    planes = np.ascontiguousarray(planes, dtype=np.float64)
    if planes.ndim == 2:
        planes = planes[None]
    if first_record < 1:
        raise ValueError("records are numbered from 1")
    recl = planes.shape[1] * planes.shape[2] * 8
    mode = "r+b" if os.path.exists(path) else "w+b"
    with open(path, mode) as f:
        f.seek((first_record - 1) * recl)
        f.write(planes.astype(np.dtype("=f8"), copy=False).tobytes())


def read_vz_cc_bin(path: str, nx: int, ny: int, nrec: int | None = None) -> np.ndarray:
    """Records 1..nrec (all whole records by default) as (nrec, ny, nx)."""
    recl = nx * ny * 8
    size = os.path.getsize(path)
    if nrec is None:
        nrec = size // recl
    if nrec * recl > size:
        raise ValueError(f"{path}: {size} bytes hold fewer than {nrec} records of {recl} bytes")
    data = np.fromfile(path, dtype=np.dtype("=f8"), count=nrec * nx * ny)
    return data.reshape(nrec, ny, nx)


# ---- FITS ----------------------------------------------------------------

def _card(key: str, value, comment: str = "") -> bytes:
    if isinstance(value, bool):
        v = "T" if value else "F"
        s = f"{key:<8}= {v:>20}"
    elif isinstance(value, (int, np.integer)):
        s = f"{key:<8}= {int(value):>20}"
    elif isinstance(value, (float, np.floating)):
        r = repr(float(value)).upper()
        if "E" not in r and "." not in r:
            r += "."
        s = f"{key:<8}= {r:>20}"
    else:
        s = f"{key:<8}= '{str(value):<8}'"
    if comment:
        s += f" / {comment}"
    if len(s) > 80:
        raise ValueError(f"FITS card too long: {s!r}")
    return s.ljust(80).encode("ascii")


def write_fits(path: str, array: np.ndarray, keywords: dict | None = None) -> None:
    """Primary array, BITPIX = -64; array (n3, ny, nx) [or (ny, nx)] gives
    NAXIS1 = nx, NAXIS2 = ny, NAXIS3 = n3.  keywords: extra (name, value)
    cards, e.g. {"TIME": time} as writefits_3D writes."""
    a = np.ascontiguousarray(array, dtype=np.float64)
    shape = a.shape[::-1]                       # NAXIS1 first
    cards = [_card("SIMPLE", True, "file does conform to FITS standard"),
             _card("BITPIX", -64, "number of bits per data pixel"),
             _card("NAXIS", len(shape), "number of data axes")]
    for i, n in enumerate(shape):
        cards.append(_card(f"NAXIS{i + 1}", int(n), f"length of data axis {i + 1}"))
    cards.append(_card("EXTEND", False))
    for k, v in (keywords or {}).items():
        cards.append(_card(k.upper(), v))
    cards.append(b"END".ljust(80))
    header = b"".join(cards)
    header += b" " * (-len(header) % FITS_BLOCK)
    data = a.astype(">f8", copy=False).tobytes()
    data += b"\0" * (-len(data) % FITS_BLOCK)
    with open(path, "wb") as f:
        f.write(header)
        f.write(data)


def read_fits(path: str, with_header: bool = False):
    """Primary array of a FITS file (BITPIX -64, -32, 8, 16, 32, 64) as a
    float64 array in C order (NAXISn ... NAXIS1), BSCALE/BZERO applied."""
    with open(path, "rb") as f:
        raw = f.read()
    hdr = {}
    pos = 0
    while True:
        if pos + FITS_BLOCK > len(raw):
            raise ValueError(f"{path}: no END card")
        block = raw[pos:pos + FITS_BLOCK]
        pos += FITS_BLOCK
        done = False
        for i in range(0, FITS_BLOCK, 80):
            card = block[i:i + 80].decode("ascii")
            key = card[:8].strip()
            if key == "END":
                done = True
                break
            if card[8:10] == "= ":
                val = card[10:].split("/")[0].strip()
                if val.startswith("'"):
                    hdr[key] = val.strip("'").rstrip()
                elif val in ("T", "F"):
                    hdr[key] = val == "T"
                else:
                    try:
                        hdr[key] = int(val)
                    except ValueError:
                        hdr[key] = float(val.replace("D", "E"))
        if done:
            break
    bitpix = int(hdr["BITPIX"])
    naxis = int(hdr["NAXIS"])
    shape = tuple(int(hdr[f"NAXIS{i}"]) for i in range(naxis, 0, -1))
    dt = {-64: ">f8", -32: ">f4", 8: ">u1", 16: ">i2", 32: ">i4", 64: ">i8"}[bitpix]
    n = int(np.prod(shape)) if shape else 0
    a = np.frombuffer(raw, dtype=dt, count=n, offset=pos).astype(np.float64).reshape(shape)
    if "BSCALE" in hdr or "BZERO" in hdr:
        a = a * float(hdr.get("BSCALE", 1.0)) + float(hdr.get("BZERO", 0.0))
    return (a, hdr) if with_header else a


# ---- text files ------------------------------------------------------------

def write_kernel_info(path: str, values) -> None:
    """One integer per line (driver.f90:307-309 forward: init, maxtime;
    :346-352 adjoint: number of source slices, last output time)."""
    with open(path, "w") as f:
        for v in values:
            f.write(f"{int(v):12d}\n")


def read_kernel_info(path: str) -> list:
    with open(path) as f:
        return [int(line.split()[0]) for line in f if line.strip()]


def write_timeline(path: str, rows) -> None:
    """``time timeline`` per output (driver.f90:457)."""
    with open(path, "w") as f:
        for t, tl in rows:
            f.write(f"{int(t):12d} {float(tl):25.16E}\n")


def read_timeline(path: str) -> np.ndarray:
    return np.loadtxt(path, ndmin=2)


# ---- the reference's output set of one run ---------------------------------

def write_forward_outputs(directory: str, p, records: np.ndarray, init: int = 0) -> dict:
    """vz_cc.bin, vz_cc.fits, timeline and kernel_info of a forward run whose
    surface records (nrec, ny, nx) were taken every p.steps steps from time
    0 (the layout of forward_srcXX_lsYY/).  The timeline starts at
    -solartime*3600 s (initialize.f90:1029) and gains one time step per step
    before the output check (driver.f90:453-457)."""
    os.makedirs(directory, exist_ok=True)
    paths = {k: os.path.join(directory, k) for k in ("vz_cc.bin", "vz_cc.fits", "timeline", "kernel_info")}
    write_vz_cc_bin(paths["vz_cc.bin"], records)
    write_fits(paths["vz_cc.fits"], records)
    ts = float(np.float32(p.timestep))
    t0 = -float(p.solartime) * 3600.0
    write_timeline(paths["timeline"], [(k * p.steps, t0 + (k * p.steps + 1) * ts) for k in range(len(records))])
    write_kernel_info(paths["kernel_info"], [init, p.maxtime])
    return paths


def write_kernels(directory: str, contrib: str, kc: np.ndarray, krho: np.ndarray, hessian: np.ndarray,
                  time: int = 0) -> dict:
    """kernel_c_XX.fits, kernel_rho_XX.fits, hessian_XX.fits (kernels.f90:465,
    532, 539), arrays (nz, ny, nx)."""
    os.makedirs(directory, exist_ok=True)
    out = {}
    for name, arr in (("kernel_c", kc), ("kernel_rho", krho), ("hessian", hessian)):
        path = os.path.join(directory, f"{name}_{contrib}.fits")
        write_fits(path, arr, {"TIME": int(time)})
        out[name] = path
    return out


def timestamp(time: int, width: int = 6) -> str:
    """The zero-padded decimal time of the reference's file names
    (convert_to_string, initialize.f90:1092-1120, timestamp_size 6)."""
    return str(int(time)).zfill(width)


def write_partial_state(directory: str, solver, time: int, forward: bool, slot: int = 0) -> list:
    """WRITE_OUT_PARTIAL_STATE (all_modules.f90:750-785, called at
    driver.f90:481,484 on the output cadence): xi (forward runs only), v and
    the last stage's acc = scr(:,:,:,4:6) of one source slot as
    <name>_<time>_partial.fits (TIME keyword, planes 1..nz), the y
    components only in 3-D.  `solver` is a Solver after a step call (field
    0..5 = a, 9..11 = scr(4..6))."""
    os.makedirs(directory, exist_ok=True)
    three_d = solver.p.ny > 1
    names = []
    if forward:
        names += [("xix", 0), ("xiz", 2)] + ([("xiy", 1)] if three_d else [])
    names += [("acc_x", 9), ("acc_z", 11), ("vx", 3), ("vz", 5)]
    if three_d:
        names += [("acc_y", 10), ("vy", 4)]
    out = []
    ts = timestamp(time)
    for name, f in names:
        path = os.path.join(directory, f"{name}_{ts}_partial.fits")
        write_fits(path, solver.field(f, slot), {"TIME": int(time)})
        out.append(path)
    return out


def _state_units():
    """diml, dimc, dimrho, dimb as the reference forms them from its REAL*4
    literals (initialize.f90:38,751-757)."""
    def r4(x):
        return float(np.float32(x))
    pi, dimc, dimrho, diml = r4(3.14159265358979), r4(1.0e6), r4(1.0e-3), r4(69598946770.0)
    dimb = (4.0 * pi * dimc ** 2.0 * dimrho) ** 0.5
    return diml, dimc, dimrho, dimb


def _full_state_layout(p):
    """(file name, state field, unit) of WRITE_OUT_FULL_STATE for the form of
    p, and the PML auxiliaries' names (all_modules.f90:623-694)."""
    diml, dimc, dimrho, dimb = _state_units()
    magnetic = p.option in (8, 10, 18)
    if p.option in (2, 8):                    # velocity forms: rho, vx, vy, vz, p (, bx, by, bz)
        fields = [("p", 4, dimrho * dimc ** 2.0), ("vy", 2, dimc), ("rho", 0, dimrho), ("vx", 1, dimc),
                  ("vz", 3, dimc)]
        if p.option == 8:
            fields += [("bx", 5, dimb), ("by", 6, dimb), ("bz", 7, dimb)]
    else:                                     # displacement forms: xi, v
        fields = [("xix", 0, diml), ("xiz", 2, diml), ("vx", 3, dimc), ("vz", 5, dimc)]
        if p.ny > 1:
            fields += [("xiy", 1, diml), ("vy", 4, dimc)]
    pml = ["psivz", "psip"] + (["psidzbx", "psidzby", "psiinductionbx", "psiinductionby"] if magnetic else [])
    return fields, pml


def write_full_state(directory: str, solver, time: int, slot: int = 0, remove_previous: bool = False) -> list:
    """WRITE_OUT_FULL_STATE (all_modules.f90:623-694): the state of one slot
    in the reference's units as <name>_<time>_full.fits, and the PML
    auxiliaries (nzpml planes) as they are.  The reference first deletes the
    directory's earlier *full* files; remove_previous=True does the same."""
    os.makedirs(directory, exist_ok=True)
    if remove_previous:
        for f in os.listdir(directory):
            if "full" in f:
                os.remove(os.path.join(directory, f))
    a, pml = solver.state(slot)
    fields, pnames = _full_state_layout(solver.p)
    ts = timestamp(time)
    out = []
    for name, f, unit in fields:
        path = os.path.join(directory, f"{name}_{ts}_full.fits")
        write_fits(path, a[f] * unit, {"TIME": int(time)})
        out.append(path)
    for i, name in enumerate(pnames):
        path = os.path.join(directory, f"{name}_{ts}_full.fits")
        write_fits(path, pml[i], {"TIME": int(time)})
        out.append(path)
    return out


def read_full_state(directory: str, solver, time: int, slot: int = 0) -> None:
    """READ_IN_INITIAL_CONDITION (all_modules.f90:530-621): the files of
    write_full_state back into the slot's state, divided by the units.  The
    reference reads xi_y and v_y even in 2-D, where it never writes them;
    here the y components are read where they exist and are zero otherwise."""
    fields, pnames = _full_state_layout(solver.p)
    ts = timestamp(time)
    a = np.zeros((solver.nf,) + solver.shape)
    for name, f, unit in fields:
        a[f] = read_fits(os.path.join(directory, f"{name}_{ts}_full.fits")).reshape(solver.shape) / unit
    pml = np.zeros((solver.npv, solver.p.nzpml, solver.p.ny, solver.p.nx))
    for i, name in enumerate(pnames):
        pml[i] = read_fits(os.path.join(directory, f"{name}_{ts}_full.fits")).reshape(pml.shape[1:])
    solver.set_state(a, pml, slot=slot)


def write_kernels_b(directory: str, contrib: str, kbx: np.ndarray, kbz: np.ndarray, kpsi: np.ndarray,
                    time: int = 0) -> dict:
    """kernel_bx_XX.fits, kernel_bz_XX.fits, kernel_vectorpsi_XX.fits of a 2-D
    magnetic run (kernels.f90:509-512; no kernel_by in 2-D), arrays (nz, 1, nx)."""
    os.makedirs(directory, exist_ok=True)
    out = {}
    for name, arr in (("kernel_bx", kbx), ("kernel_bz", kbz), ("kernel_vectorpsi", kpsi)):
        path = os.path.join(directory, f"{name}_{contrib}.fits")
        write_fits(path, arr, {"TIME": int(time)})
        out[name] = path
    return out


def write_adjoint_source(directory: str, adj: np.ndarray, t1_min: float, tn_min: float, time: int = 0,
                         two_d: bool = True) -> dict:
    """adjoint_srcXX/source.fits (writefits_3D of adj, (nt, 1, nx) or
    (nt, nx); TIME = the time step at writing) and adjoint_srcXX/information
    (nt, t(1)*60, t(nt)*60 and '2D' for a 2-D run; driver.f90:1647-1660)."""
    os.makedirs(directory, exist_ok=True)
    a = np.asarray(adj, dtype=np.float64)
    if a.ndim == 2:
        a = a[:, None, :]
    paths = {"source.fits": os.path.join(directory, "source.fits"),
             "information": os.path.join(directory, "information")}
    write_fits(paths["source.fits"], a, {"TIME": int(time)})
    with open(paths["information"], "w") as f:
        f.write(f"{a.shape[0]:12d}\n{t1_min * 60.0:25.16E}\n{tn_min * 60.0:25.16E}\n")
        if two_d:
            f.write(" 2D\n")
    return paths


def write_misfit(path: str, index: int, nmeas: int, misfit: float) -> None:
    """kernel/misfit_XX_YY: source index, number of measurements and
    0.5 sum tau^2 on one line (driver.f90:1664-1674)."""
    with open(path, "w") as f:
        f.write(f"{int(index):12d}{int(nmeas):12d}{float(misfit):25.16E}\n")


def write_windows(directory: str, windows: dict) -> list:
    """windows.0 / windows.1 (driver.f90:1310-1325, 1489-1491): one `lef rig`
    line per measurement of the f and p1 sets in pixel order; `windows` maps
    set -> {pixel: (lef, rig)} as Solver.adjoint_source returns it."""
    os.makedirs(directory, exist_ok=True)
    out = []
    for m in (0, 1):
        path = os.path.join(directory, f"windows.{m}")
        with open(path, "w") as f:
            for i in sorted(windows.get(m, {})):
                lef, rig = windows[m][i]
                f.write(f"{int(lef):12d}{int(rig):12d}\n")
        out.append(path)
    return out


def read_windows(directory: str, pixels: dict) -> dict:
    """windows.0 / windows.1 back into set -> {pixel: (lef, rig)}; the
    reference reads the lines in the order it measures, so `pixels` gives,
    per set, the pixels in measurement order."""
    out = {}
    for m in (0, 1):
        path = os.path.join(directory, f"windows.{m}")
        if not os.path.exists(path):
            continue
        with open(path) as f:
            rows = [tuple(int(v) for v in line.split()[:2]) for line in f if line.strip()]
        out[m] = dict(zip(pixels.get(m, []), rows))
    return out
