"""The committed fixture of the reference's shipped configuration
(tests/golden/shipped_inputs.npz): its values, and, where the reference is
mounted, that make_shipped.py still reproduces it from the reference's files."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
REF = "/root/reference"


def test_shipped_fixture_values():
    from golden.make_shipped import load
    d = load()
    p = d["params"]
    assert (p.nx, p.ny, p.nz) == (256, 1, 300) and p.xlength == 400e8 and p.timestep == 2.0
    assert p.option == 18 and d["adjoint_option"] == 18          # magnetic + '2D'
    assert (p.npmlbot, p.npmltop) == (10, 0) and p.solartime == 2.0
    assert p.maxtime == 4185
    t = d["polytrope"]
    assert t.shape == (300, 6) and np.all(np.diff(t[:, 0]) > 0)
    assert d["x00"] == -5.0
    assert d["ridges"][0] == (10.0, 80.0, 10.0) and d["ridges"][1] == (20.0, 100.0, 10.0)
    assert d["bands"][0] == (1.0, 4.0) and d["bands"][1] == (2.0, 5.0)


@pytest.mark.skipif(not os.path.isdir(REF), reason="the reference is not mounted here")
def test_fixture_reproduces_from_the_reference(tmp_path):
    from golden.make_shipped import load, read_shipped, write
    out = str(tmp_path / "shipped.npz")
    write(read_shipped(REF), out)
    a, b = load(out), load()
    assert a["params"] == b["params"] and a["adjoint_option"] == b["adjoint_option"]
    assert np.array_equal(a["polytrope"], b["polytrope"])
    assert a["ridges"] == b["ridges"] and a["bands"] == b["bands"] and a["x00"] == b["x00"]
