"""GPU test of sparc_gpu_spec_to_phys_noalloc, the transform that allocates
nothing (for callers whose memory pool owns the rest of HBM, or that must not
let cudaMalloc/cudaFree synchronise the device).  It must give the same
planes as the library's existing path, on two calls in a row (the second call
runs on whatever the first left in the shared scratch array), and reject a
request beyond its scratch limit.  The file name sorts last so that a run
stopping at the first failure has already run every other test."""
import ctypes

import numpy as np
import pytest

from cases import rel_l2, small_params, table_for

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision,tol", [("f64", 1e-12), ("f32", 1e-5)])
def test_noalloc_transform_matches_existing_path(gpu_lib, precision, tol):
    import torch
    from sparc_gb300 import native
    from sparc_gb300.solver import Solver

    L = native.load()
    p = small_params(precision=precision)
    s = Solver(p, table_for(p))
    rng = np.random.default_rng(2024)
    cdt = torch.complex128 if precision == "f64" else torch.complex64
    rdt = torch.float64 if precision == "f64" else torch.float32
    for call in range(2):
        field = rng.standard_normal((p.nz, p.ny, p.nx))
        # existing entry points: physical field -> library state -> physical field
        a = np.zeros((6,) + s.shape)
        a[0] = field
        s.set_state(a)
        ref = s.field(0)
        # the same planes in the library's spectral form, in caller-owned device memory
        spec = np.fft.rfft2(field) / (p.nx * p.ny)
        d_spec = torch.from_numpy(np.ascontiguousarray(spec)).to(device="cuda", dtype=cdt)
        d_phys = torch.full((p.nz, p.ny, p.nx), float("nan"), dtype=rdt, device="cuda")
        torch.cuda.synchronize()
        rc = L.sparc_gpu_spec_to_phys_noalloc(s.h, ctypes.c_void_p(d_spec.data_ptr()),
                                               ctypes.c_void_p(d_phys.data_ptr()), p.nz, None)
        assert rc == native.SPARC_OK, L.sparc_gpu_last_error(s.h)
        s.sync()
        torch.cuda.synchronize()
        out = d_phys.double().cpu().numpy()
        assert np.all(np.isfinite(out)), call
        assert rel_l2(out, ref) < tol, (call, rel_l2(out, ref))
    s.close()


def test_noalloc_rejects_requests_beyond_the_scratch_limit(gpu_lib):
    import torch
    from sparc_gb300 import native
    from sparc_gb300.solver import Solver

    L = native.load()
    p = small_params()
    s = Solver(p, table_for(p))
    per_plane = p.ny * (p.nx // 2 + 1) * 16
    limit = (32 << 20) // per_plane
    d = torch.zeros(16, dtype=torch.float64, device="cuda")
    rc = L.sparc_gpu_spec_to_phys_noalloc(s.h, ctypes.c_void_p(d.data_ptr()), ctypes.c_void_p(d.data_ptr()),
                                           limit + 1, None)
    assert rc == native.SPARC_EINVAL
    msg = L.sparc_gpu_last_error(s.h).decode()
    assert "no-allocation limit" in msg and f"at most {limit} planes" in msg
    assert L.sparc_gpu_spec_to_phys_noalloc(s.h, None, None, 1, None) == native.SPARC_EINVAL
    s.close()
