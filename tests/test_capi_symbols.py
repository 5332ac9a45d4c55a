"""The C-ABI library builds for sm_103a, loads without a GPU and exports every
function that include/sparc_gpu.h declares (no compute calls here)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    txt = open(os.path.join(ROOT, "include", "sparc_gpu.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(sparc_gpu_\w+)\s*\(", txt)))


@pytest.fixture(scope="module")
def lib():
    from sparc_gb300 import build
    path = build.build()
    return ctypes.CDLL(path)


def test_every_declared_function_is_exported(lib):
    names = header_functions()
    assert len(names) >= 30
    for n in names:
        assert hasattr(lib, n), n


def test_binding_covers_header():
    from sparc_gb300 import native
    assert sorted(native.EXPORTS) == header_functions()


def test_host_only_calls(lib):
    from sparc_gb300 import native
    L = native.load()
    assert L.sparc_gpu_abi_version() == 1
    assert L.sparc_gpu_errstr(0) == b"ok"
    assert L.sparc_gpu_errstr(native.SPARC_EIO).startswith(b"file")
    h = ctypes.c_void_p()
    assert L.sparc_gpu_create(None, ctypes.byref(h)) == native.SPARC_EINVAL
    bad = native.CParams(nx=100, ny=100, nz=10)
    assert L.sparc_gpu_create(ctypes.byref(bad), ctypes.byref(h)) == native.SPARC_EINVAL
    assert not h.value
    L.sparc_gpu_destroy(None)


def test_missing_library_fails_loudly(tmp_path, monkeypatch):
    from sparc_gb300 import native
    monkeypatch.setattr(native, "_lib", None)
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        native.load(str(tmp_path / "nope.so"))


def test_table_row_counts_match_header():
    """The binding sizes the diagnostic tables from the header's row counts."""
    import re
    from sparc_gb300 import native
    hdr = open(os.path.join(os.path.dirname(__file__), "..", "include", "sparc_gpu.h")).read()
    rows = dict(re.findall(r"#define (SPARC_[ZP]TAB_ROWS) (\d+)", hdr))
    assert int(rows["SPARC_ZTAB_ROWS"]) == native.ZTAB_ROWS
    assert int(rows["SPARC_PTAB_ROWS"]) == native.PTAB_ROWS


def test_binding_argument_counts_match_header():
    """Every prototype of include/sparc_gpu.h has as many parameters as the
    ctypes binding declares for it (argtypes), so a changed signature cannot
    be called with a stale one."""
    from sparc_gb300 import native
    txt = open(os.path.join(ROOT, "include", "sparc_gpu.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    protos = dict((m.group(1), m.group(2)) for m in
                  re.finditer(r"\b(sparc_gpu_\w+)\s*\(([^;{]*?)\)\s*;", txt, flags=re.S))
    L = native.load()
    checked = 0
    for name, params in protos.items():
        f = getattr(L, name)
        if f.argtypes is None:
            continue
        p = params.strip()
        n = 0 if p in ("", "void") else len(p.split(","))
        assert n == len(f.argtypes), (name, n, len(f.argtypes))
        checked += 1
    assert checked >= 30
