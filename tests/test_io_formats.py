"""The reference's on-disk formats (vz_cc.bin, FITS BITPIX -64, kernel_info,
timeline): layout checks and round trips, no GPU."""
import os

import numpy as np

from sparc_gb300 import io
from sparc_gb300.params import SparcParams


def test_vz_cc_bin_is_fixed_records_x_fastest(tmp_path):
    nx, ny = 6, 4
    rec = np.arange(3 * ny * nx, dtype=np.float64).reshape(3, ny, nx)
    path = str(tmp_path / "vz_cc.bin")
    io.write_vz_cc_bin(path, rec)
    raw = np.fromfile(path, dtype="=f8")
    assert raw.size == 3 * nx * ny
    # record k (1-based) at byte offset (k-1)*nx*ny*8, element (i, j) at j*nx + i
    assert raw[1 * nx * ny + 2 * nx + 5] == rec[1, 2, 5]
    # appending records as write_binary_seq_2D does, one per output
    io.write_vz_cc_bin(path, rec[0] * -1.0, first_record=4)
    back = io.read_vz_cc_bin(path, nx, ny)
    assert back.shape == (4, ny, nx)
    assert np.array_equal(back[:3], rec) and np.array_equal(back[3], -rec[0])


def test_fits_header_and_data_layout(tmp_path):
    a = np.random.default_rng(0).standard_normal((5, 3, 7))
    path = str(tmp_path / "k.fits")
    io.write_fits(path, a, {"TIME": 7200})
    raw = open(path, "rb").read()
    assert len(raw) % 2880 == 0
    cards = [raw[i:i + 80].decode() for i in range(0, 2880, 80)]
    assert cards[0].startswith("SIMPLE  =                    T")
    assert cards[1].startswith("BITPIX  =                  -64")
    assert cards[2].startswith("NAXIS   =                    3")
    assert cards[3].startswith("NAXIS1  =                    7")     # nx first
    assert cards[4].startswith("NAXIS2  =                    3")
    assert cards[5].startswith("NAXIS3  =                    5")
    assert any(c.startswith("TIME    =                 7200") for c in cards)
    assert any(c.rstrip() == "END" for c in cards)
    data = np.frombuffer(raw, dtype=">f8", count=a.size, offset=2880)
    assert np.array_equal(data, a.ravel())                           # x fastest, big endian
    back, hdr = io.read_fits(path, with_header=True)
    assert np.array_equal(back, a) and hdr["TIME"] == 7200 and hdr["BITPIX"] == -64


def test_fits_reads_float32_and_scaled(tmp_path):
    a = np.arange(12, dtype=np.float32).reshape(3, 4)
    hdr = b"".join([io._card("SIMPLE", True), io._card("BITPIX", -32), io._card("NAXIS", 2),
                    io._card("NAXIS1", 4), io._card("NAXIS2", 3), io._card("BSCALE", 2.0),
                    io._card("BZERO", 1.0), b"END".ljust(80)])
    hdr += b" " * (-len(hdr) % 2880)
    path = tmp_path / "f.fits"
    path.write_bytes(hdr + a.astype(">f4").tobytes())
    assert np.array_equal(io.read_fits(str(path)), a * 2.0 + 1.0)


def test_forward_output_set(tmp_path):
    p = SparcParams(nx=8, ny=4, nz=20, solartime=1.0)
    rec = np.random.default_rng(1).standard_normal((5, 4, 8))
    paths = io.write_forward_outputs(str(tmp_path), p, rec)
    assert np.array_equal(io.read_vz_cc_bin(paths["vz_cc.bin"], 8, 4), rec)
    assert np.array_equal(io.read_fits(paths["vz_cc.fits"]), rec)
    tl = io.read_timeline(paths["timeline"])
    assert tl.shape == (5, 2)
    assert tl[0, 0] == 0 and tl[1, 0] == p.steps
    assert tl[0, 1] == -3600.0 + p.timestep and tl[2, 1] == -3600.0 + (2 * p.steps + 1) * p.timestep
    assert io.read_kernel_info(paths["kernel_info"]) == [0, p.maxtime]
    k = io.write_kernels(str(tmp_path), "01", rec, 2 * rec, 3 * rec, time=p.maxtime)
    assert np.array_equal(io.read_fits(k["kernel_rho"]), 2 * rec)


def test_magnetic_kernel_files(tmp_path):
    """kernel_bx / kernel_bz / kernel_vectorpsi (kernels.f90:509-512): FITS
    BITPIX -64 with NAXIS2 = 1 for the 2-D box and the TIME keyword."""
    k = np.random.default_rng(2).standard_normal((3, 12, 1, 16))
    paths = io.write_kernels_b(str(tmp_path), "03", k[0], k[1], k[2], time=4185)
    assert sorted(os.path.basename(v) for v in paths.values()) == [
        "kernel_bx_03.fits", "kernel_bz_03.fits", "kernel_vectorpsi_03.fits"]
    a, hdr = io.read_fits(paths["kernel_vectorpsi"], with_header=True)
    assert np.array_equal(a, k[2])
    assert (hdr["NAXIS1"], hdr["NAXIS2"], hdr["NAXIS3"], hdr["TIME"], hdr["BITPIX"]) == (16, 1, 12, 4185, -64)


def test_adjoint_source_files(tmp_path):
    adj = np.random.default_rng(4).standard_normal((30, 16))
    paths = io.write_adjoint_source(str(tmp_path / "adjoint_src01"), adj, 0.25, 14.75, time=1799)
    a, hdr = io.read_fits(paths["source.fits"], with_header=True)
    assert a.shape == (30, 1, 16) and np.array_equal(a[:, 0], adj) and hdr["TIME"] == 1799
    lines = open(paths["information"]).read().split()
    assert int(lines[0]) == 30 and float(lines[1]) == 15.0 and float(lines[2]) == 885.0 and lines[3] == "2D"
    io.write_misfit(str(tmp_path / "misfit_01_00"), 1, 42, 0.125)
    assert open(tmp_path / "misfit_01_00").read().split() == ["1", "42", "1.2500000000000000E-01"]
    win = {0: {5: (10, 50), 3: (8, 48)}, 1: {7: (20, 50)}}
    io.write_windows(str(tmp_path), win)
    back = io.read_windows(str(tmp_path), {0: [3, 5], 1: [7]})
    assert back == {0: {3: (8, 48), 5: (10, 50)}, 1: {7: (20, 50)}}


def test_partial_state_files(tmp_path):
    """WRITE_OUT_PARTIAL_STATE's names, fields and TIME keyword, from any
    object with the Solver's field accessor."""
    import numpy as np
    from sparc_gb300 import io
    from sparc_gb300.params import SparcParams

    class FakeSolver:
        def __init__(self, p):
            self.p = p

        def field(self, f, slot=0):
            return np.full((self.p.nz, self.p.ny, self.p.nx), float(f * 10 + slot))

    p3 = SparcParams(nx=8, ny=8, nz=16)
    files = io.write_partial_state(str(tmp_path / "fwd"), FakeSolver(p3), 1234, forward=True, slot=1)
    names = sorted(f.split("/")[-1] for f in files)
    assert names == sorted(f"{n}_001234_partial.fits" for n in
                           ("xix", "xiz", "xiy", "acc_x", "acc_z", "vx", "vz", "acc_y", "vy"))
    a, hdr = io.read_fits(str(tmp_path / "fwd" / "acc_z_001234_partial.fits"), with_header=True)
    assert a.shape == (16, 8, 8) and np.all(a == 111.0) and int(hdr["TIME"]) == 1234
    p2 = SparcParams(nx=8, ny=1, nz=16, option=17)
    files = io.write_partial_state(str(tmp_path / "adj"), FakeSolver(p2), 45, forward=False)
    assert sorted(f.split("/")[-1] for f in files) == sorted(
        f"{n}_000045_partial.fits" for n in ("acc_x", "acc_z", "vx", "vz"))


def test_full_state_round_trip(tmp_path):
    """WRITE_OUT_FULL_STATE / READ_IN_INITIAL_CONDITION: names, units and a
    round trip through the files, for the displacement, velocity and MHD
    forms, with a stand-in of the Solver's state accessors."""
    import numpy as np
    from sparc_gb300 import io
    from sparc_gb300.params import SparcParams

    class FakeSolver:
        def __init__(self, p, nf, npv, seed):
            self.p, self.nf, self.npv = p, nf, npv
            self.shape = (p.nz, p.ny, p.nx)
            rng = np.random.default_rng(seed)
            self.a = rng.standard_normal((nf,) + self.shape)
            self.pml = rng.standard_normal((npv, p.nzpml, p.ny, p.nx))
            self.got = None

        def state(self, slot=0):
            return self.a, self.pml

        def set_state(self, a, pml, slot=0):
            self.got = (a, pml)

    diml, dimc, dimrho, dimb = io._state_units()
    for opt, ny, nf, npv, names in ((4, 8, 6, 2, ("xix", "xiy", "xiz", "vx", "vy", "vz", "psivz", "psip")),
                                    (17, 1, 6, 2, ("xix", "xiz", "vx", "vz", "psivz", "psip")),
                                    (8, 8, 8, 6, ("rho", "vx", "vy", "vz", "p", "bx", "by", "bz", "psivz",
                                                  "psip", "psidzbx", "psidzby", "psiinductionbx",
                                                  "psiinductionby"))):
        p = SparcParams(nx=8, ny=ny, nz=16, option=opt, npmlbot=3, npmltop=3)
        src = FakeSolver(p, nf, npv, opt)
        d = tmp_path / f"opt{opt}"
        files = io.write_full_state(str(d), src, 30, slot=0)
        assert sorted(f.split("/")[-1] for f in files) == sorted(f"{n}_000030_full.fits" for n in names)
        dst = FakeSolver(p, nf, npv, 99)
        io.read_full_state(str(d), dst, 30)
        a, pml = dst.got
        used = [f for _, f, _ in io._full_state_layout(p)[0]]
        assert np.allclose(a[used], src.a[used], rtol=1e-15, atol=0) and np.array_equal(pml, src.pml)
    first = io.read_fits(str(tmp_path / "opt4" / "xix_000030_full.fits"))
    assert np.allclose(first, FakeSolver(SparcParams(nx=8, ny=8, nz=16, option=4, npmlbot=3, npmltop=3), 6, 2, 4).a[0] * diml,
                       rtol=1e-15, atol=0)
