"""Cross-check of the hand-written transforms against cuFFT (through
torch.fft on the GPU): the library's FP64 d/dx and d/dy (derivatives.f90:
28-170: r2c, times i k with the reference's REAL*4 pi and stretch, Nyquist
dropped, c2r) against the same multipliers applied to cuFFT spectra.  cuFFT
is the check only; the library does not call it."""
import numpy as np
import pytest

from cases import rel_l2, small_params, table_for

pytestmark = pytest.mark.gpu


def _r4(x):
    return float(np.float32(x))


def _multipliers(p, n, length):
    """i k stretch of derivatives.f90 for an axis of n points, the reference's
    REAL*4 literals (pi, R_sun, the box length), Nyquist set to zero."""
    pi = _r4(3.14159265358979)
    stretch = _r4(69598946770.0) / _r4(length)
    k = np.fft.fftfreq(n) * n
    m = k * (1.0 / n) * 2.0 * pi * n * stretch
    if n % 2 == 0:
        m[n // 2] = 0.0
    return m


@pytest.mark.parametrize("nx,ny,nz", [(256, 256, 16), (64, 32, 16), (512, 16, 16)])
def test_derivatives_against_cufft(gpu_lib, nx, ny, nz):
    torch = pytest.importorskip("torch")
    from sparc_gb300.solver import Solver
    p = small_params(nx=nx, ny=ny, nz=nz, npmlbot=3, npmltop=3, precision="f64")
    rng = np.random.default_rng(nx + ny)
    v = rng.standard_normal((nz, ny, nx))
    with Solver(p, table_for(p)) as s:
        dx = s.ddx(v)
        dy = s.ddy(v)
    t = torch.from_numpy(v).cuda()
    mx = torch.from_numpy(_multipliers(p, nx, p.xlength)[: nx // 2 + 1]).cuda()
    my = torch.from_numpy(_multipliers(p, ny, p.ylength)).cuda()
    ref_x = torch.fft.irfft(torch.fft.rfft(t, dim=-1) * (1j * mx), n=nx, dim=-1).cpu().numpy()
    ref_y = torch.fft.ifft(torch.fft.fft(t, dim=-2) * (1j * my)[:, None], dim=-2).real.cpu().numpy()
    assert np.abs(ref_x).max() > 0
    assert rel_l2(dx, ref_x) < 1e-12, rel_l2(dx, ref_x)
    assert rel_l2(dy, ref_y) < 1e-12, rel_l2(dy, ref_y)
