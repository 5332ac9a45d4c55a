"""A C program drives the library through include/sparc_gpu.h in the call
order of the reference's TIMESTEPPING loop (create -> set_background ->
set_source -> step / get_field at the output cadence -> destroy).  On the CPU
it must compile and link; on the GPU its surface records must equal the
records of the same run through the Python binding bit for bit, and match the
oracle's to 1e-10."""
import os
import subprocess
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "c_harness"))


def test_c_harness_compiles_and_links(tmp_path):
    import build as hb
    exe = hb.build(str(tmp_path))
    assert os.access(exe, os.X_OK)


@pytest.mark.gpu
def test_c_harness_records_match_binding_and_oracle(tmp_path, gpu_lib):
    import build as hb
    from cases import gaussian_plane, rel_l2, small_params, table_for
    from oracle import oracle as O
    from sparc_gb300.background import write_polytrope
    from sparc_gb300.solver import Solver
    exe = hb.build(str(tmp_path))
    p = small_params()                         # the harness's fixed constants are small_params'
    tab = table_for(p)
    plane = gaussian_plane(p)
    series = O.forward_source(p, 200) * 1e3
    write_polytrope(str(tmp_path / "bg.txt"), tab)
    tab = np.loadtxt(str(tmp_path / "bg.txt"))     # the harness reads the printed table
    plane.astype(np.float64).tofile(str(tmp_path / "plane.bin"))
    series.astype(np.float64).tofile(str(tmp_path / "series.bin"))
    nsteps = 46
    r = subprocess.run([exe, str(p.nx), str(p.ny), str(p.nz), repr(p.xlength), str(p.npmlbot), str(p.npmltop),
                        "0", str(nsteps), str(tmp_path / "bg.txt"), str(tmp_path / "plane.bin"),
                        str(tmp_path / "series.bin"), str(tmp_path / "out.bin")],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    recs = np.fromfile(str(tmp_path / "out.bin")).reshape(-1, p.ny, p.nx)
    assert recs.shape[0] == 4 and np.abs(recs).max() > 0
    s = Solver(p, tab)
    s.set_source_series(plane, series)
    s.record_surface(8)
    s.step(nsteps)
    assert np.array_equal(s.records(), recs)
    o = O.Oracle(p, tab)
    o.set_source(1, plane[None].copy(), series)
    orad = int(o.info()["o_rad"])
    ref = []
    for i in range(nsteps):
        o.step(1)
        if i % p.steps == 0:
            ref.append(o.state()[0][5, orad - 1].copy())
    assert rel_l2(recs, np.array(ref)) < 1e-10
