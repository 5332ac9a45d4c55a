// SPARC time-stepping path -- CPU FP64 ORACLE (test infrastructure only).
//
// This file is a line-for-line restatement, in C++17, of the reference Fortran
// path (jishnub/sparc).  It exists to check the GPU product, to generate the
// golden fixtures under tests/golden/, and to time a CPU baseline.  It is never
// linked into, loaded by, or called from the product library.
//
// Parity status: UNPINNED.  The reference ships no tests, fixtures or golden
// vectors, and it cannot be compiled here (no Fortran compiler, no MPI, no
// FFTW, no CFITSIO).  The restatement is pinned only by known-answer tests that
// follow from the reference's own coefficients (tests/test_oracle_kat.py).
//
// Reference literals: the reference makefile has no -r8/-fdefault-real-8, so
// every real literal without a d-exponent is a 4-byte REAL.  Constants such as
// pi (initialize.f90:38), rsun (initialize.f90:38), the LDDRK optimals
// (step.f90:28-32), the compact-FD boundary coefficients (dbyd2.f90:104-159)
// and the decay coefficients (initialize.f90:215-221) therefore carry
// single-precision rounding even though they are stored in REAL*8.  R4() below
// reproduces that rounding.
//
// Array layout: Fortran column-major (x fastest, then y, then z), i.e. the
// element (i,j,k) (1-based in Fortran) lives at (i-1) + nx*((j-1) + ny*(k-1)).

#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#include <stdexcept>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef std::complex<double> cplx;

static inline double R4(double x) { return (double)(float)x; }

// ----------------------------------------------------------------------------
// parameters (mirrors params.i + the Instruction-file flags)
// ----------------------------------------------------------------------------
extern "C" {
typedef struct {
    int nx, ny, nz;
    int npmlbot, npmltop;
    int option;           // 4 = MP_QUIET_PML_3D_DISPL, 17 = MP_QUIET_PML_2D_DISPL
    int compute_forward;  // kernel-mode roles (initialize.f90:1013-1045)
    int compute_adjoint;
    int damp_waves;       // params.i:38
    int src_k;            // 1-based source plane override (0 = use e_rad / o_rad)
    int reserved;
    double xlength, ylength, timestep;   // params.i:26-27 (cgs, seconds)
    double excitdep, obsheight;          // params.i:130,150
    double cadforcing, outputcad;        // params.i:47,136
    double nupeak, nuwidth;              // params.i:64
    double solartime;                    // params.i:129
} oracle_params;
}

// ----------------------------------------------------------------------------
// FFT (own radix-2 complex transform; FFTW semantics are restated on top)
// ----------------------------------------------------------------------------
static void fft_inplace(cplx* a, int n, int sign) {
    if (n == 1) return;
    // bit reversal
    for (int i = 1, j = 0; i < n; ++i) {
        int bit = n >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) std::swap(a[i], a[j]);
    }
    for (int len = 2; len <= n; len <<= 1) {
        int half = len >> 1;
        for (int k = 0; k < half; ++k) {
            double ang = sign * 2.0 * M_PI * k / len;
            cplx w(std::cos(ang), std::sin(ang));
            for (int i = 0; i < n; i += len) {
                cplx u = a[i + k], v = a[i + k + half] * w;
                a[i + k] = u + v;
                a[i + k + half] = u - v;
            }
        }
    }
}

// FFTW r2c (unnormalised, e^{-i}): in[n] -> out[n/2+1]
static void r2c(const double* in, long stride, int n, cplx* out, std::vector<cplx>& work) {
    work.resize(n);
    for (int i = 0; i < n; ++i) work[i] = cplx(in[i * stride], 0.0);
    fft_inplace(work.data(), n, -1);
    for (int k = 0; k <= n / 2; ++k) out[k] = work[k];
}

// FFTW c2r (unnormalised, e^{+i}): in[n/2+1] -> out[n].  The imaginary parts of
// the DC and (even n) Nyquist inputs do not contribute, as in FFTW.
static void c2r(const cplx* in, int n, double* out, long stride, std::vector<cplx>& work) {
    work.resize(n);
    if (n == 1) { out[0] = in[0].real(); return; }
    work[0] = cplx(in[0].real(), 0.0);
    for (int k = 1; k < n / 2; ++k) {
        work[k] = in[k];
        work[n - k] = std::conj(in[k]);
    }
    work[n / 2] = cplx(in[n / 2].real(), 0.0);
    fft_inplace(work.data(), n, +1);
    for (int i = 0; i < n; ++i) out[i * stride] = work[i].real();
}

// ----------------------------------------------------------------------------
// MTRIDAG, ISPECIAL=0 branch (mtridag.f90:94-111)
// r and u may alias.  Arrays a,b,c are 1-based in the reference; here 0-based.
// ----------------------------------------------------------------------------
static void mtridag0(const double* A, const double* B, const double* C,
                     double* R, long N1, int N2) {
    std::vector<double> gam(N2), betad(N2);
    betad[0] = B[0];
    for (int J = 1; J < N2; ++J) {            // mtridag.f90:96-99
        gam[J] = C[J - 1] / betad[J - 1];
        betad[J] = B[J] - A[J] * gam[J];
    }
#pragma omp parallel
    {
        std::vector<double> ud(N2);
#pragma omp for schedule(static)
        for (long I = 0; I < N1; ++I) {        // mtridag.f90:100-111
            ud[0] = R[I] / betad[0];
            for (int J = 1; J < N2; ++J)
                ud[J] = (R[I + N1 * (long)J] - A[J] * ud[J - 1]) / betad[J];
            for (int J = N2 - 2; J >= 0; --J)
                ud[J] = ud[J] - gam[J + 1] * ud[J + 1];
            for (int J = 0; J < N2; ++J) R[I + N1 * (long)J] = ud[J];
        }
    }
}

// MTRIDAG, ISPECIAL=1 (periodic) branch (mtridag.f90:19-64)
static void mtridag1(const double* a, const double* b, const double* c,
                     double* R, long N1, int n2) {
    std::vector<double> betad(n2), betas(n2), betau(n2), alpha(n2), alphab(n2);
    for (int i = 0; i < n2; ++i) {
        betad[i] = b[i]; betas[i] = 0; betau[i] = c[i]; alpha[i] = a[i]; alphab[i] = 0;
    }
    betas[0] = a[0];
    betas[n2 - 2] = c[n2 - 2];
    alphab[0] = c[n2 - 1];
    alphab[n2 - 2] = a[n2 - 1];
    for (int i = 1; i < n2 - 1; ++i) {
        betad[i] = betad[i] - alpha[i - 1] * betau[i - 1];
        betas[i] = betas[i] - alpha[i - 1] * betas[i - 1];
        alpha[i] = alpha[i] / betad[i];
        alphab[i] = (alphab[i] - alphab[i - 1] * betau[i - 1]) / betad[i];
    }
    for (int i = 0; i < n2 - 1; ++i) betad[n2 - 1] = betad[n2 - 1] - alphab[i] * betas[i];
#pragma omp parallel
    {
        std::vector<double> ud(n2);
#pragma omp for schedule(static)
        for (long I = 0; I < N1; ++I) {
            ud[0] = R[I];
            for (int j = 1; j < n2 - 1; ++j) ud[j] = R[I + N1 * (long)j] - alpha[j - 1] * ud[j - 1];
            ud[n2 - 1] = R[I + N1 * (long)(n2 - 1)];
            for (int j = 0; j < n2 - 1; ++j) ud[n2 - 1] = ud[n2 - 1] - alphab[j] * ud[j];
            ud[n2 - 1] = ud[n2 - 1] / betad[n2 - 1];
            ud[n2 - 2] = (ud[n2 - 2] - betau[n2 - 2] * ud[n2 - 1]) / betad[n2 - 2];
            for (int j = n2 - 3; j >= 0; --j)
                ud[j] = (ud[j] - betau[j] * ud[j + 1] - betas[j] * ud[n2 - 1]) / betad[j];
            for (int j = 0; j < n2; ++j) R[I + N1 * (long)j] = ud[j];
        }
    }
}

// ----------------------------------------------------------------------------
// DBYD2 (dbyd2.f90:8-237): sixth-order compact first derivative of B along its
// second index, stored in A.  For ibc = 2 / 3 / 4 the caller pre-sets A(:,1)
// and/or A(:,N2) (dbyd2.f90:130,140).
// ----------------------------------------------------------------------------
extern "C" int oracle_dbyd2(double* A, const double* B, long N1, int N2, int ibc) {
    if (ibc < 0) { A[0] = 1.0; return 0; }          // dbyd2.f90:36-39
    if (ibc > 5) return -1;                          // dbyd2.f90:40-43 (stop)
    double d2i = (ibc == 5) ? (double)(float)N2 : (double)(float)(N2 - 1);  // :46-50
    auto Bv = [&](long i, int j) { return B[i + N1 * (long)j]; };
    auto Av = [&](long i, int j) -> double& { return A[i + N1 * (long)j]; };
    if (N2 < 5) {                                    // dbyd2.f90:53-87
        for (int j = 0; j < N2; ++j)
            for (long i = 0; i < N1; ++i) {
                if (ibc == 0) Av(i, j) = 0.0;
                else if (ibc == 1) Av(i, j) = Bv(i, N2 - 1) - Bv(i, 0);
                else if (ibc == 2) Av(i, j) = Av(i, 0);
                else if (ibc == 3) Av(i, j) = Av(i, N2 - 1);
                else if (ibc == 4) Av(i, j) = ((double)(float)j * Av(i, 0) + (double)(float)(N2 - 1 - j) * Av(i, N2 - 1)) / d2i;
            }
        return 0;
    }
    double C1 = d2i * 7.0 / 9.0;                     // dbyd2.f90:88-89
    double C2 = d2i / 36.0;
    std::vector<double> uppr(N2 + 1, 0.0), lowr(N2 + 1, 0.0), diag(N2 + 1, 1.0);  // 1-based
#pragma omp parallel for schedule(static)
    for (int I = 3; I <= N2 - 2; ++I)                // dbyd2.f90:94-99 (every ibc)
        for (long J = 0; J < N1; ++J)
            Av(J, I - 1) = C1 * (Bv(J, I) - Bv(J, I - 2)) + C2 * (Bv(J, I + 1) - Bv(J, I - 3));
    if (ibc < 5) {
        // fourth-order near-boundary rows (dbyd2.f90:104-118); REAL*4 ratios
        C1 = -(double)(43.0f / 96.0f) * d2i;
        C2 = -(double)(5.0f / 6.0f) * d2i;
        double C3 = (double)(9.0f / 8.0f) * d2i;
        double C4 = (double)(1.0f / 6.0f) * d2i;
        double C5 = -(double)(1.0f / 96.0f) * d2i;
        for (long I = 0; I < N1; ++I)
            Av(I, 1) = C1 * Bv(I, 0) + C2 * Bv(I, 1) + C3 * Bv(I, 2) + C4 * Bv(I, 3) + C5 * Bv(I, 4);
        for (long I = 0; I < N1; ++I)
            Av(I, N2 - 2) = -(C1 * Bv(I, N2 - 1) + C2 * Bv(I, N2 - 2) + C3 * Bv(I, N2 - 3) +
                              C4 * Bv(I, N2 - 4) + C5 * Bv(I, N2 - 5));
        // fifth-order boundary rows (dbyd2.f90:122-146)
        C1 = -(double)(10.0f / 3.0f) * d2i;
        C2 = -3.0 * d2i;
        C3 = 6.0 * d2i;
        C4 = (double)(1.0f / 3.0f) * d2i;
        if (ibc == 0) {
            for (long I = 0; I < N1; ++I) Av(I, 0) = 0.0;
        } else if (ibc == 1 || ibc == 3) {
            for (long I = 0; I < N1; ++I)
                Av(I, 0) = C1 * Bv(I, 0) + C2 * Bv(I, 1) + C3 * Bv(I, 2) + C4 * Bv(I, 3);
        }
        if (ibc == 0) {
            for (long I = 0; I < N1; ++I) Av(I, N2 - 1) = 0.0;
        } else if (ibc == 1 || ibc == 2) {
            for (long I = 0; I < N1; ++I)
                Av(I, N2 - 1) = -(C1 * Bv(I, N2 - 1) + C2 * Bv(I, N2 - 2) + C3 * Bv(I, N2 - 3) + C4 * Bv(I, N2 - 4));
        }
        // matrix (dbyd2.f90:152-196)
        double alpha = (double)(1.0f / 3.0f);
        for (int J = 3; J <= N2 - 2; ++J) uppr[J] = alpha;
        double alpha2 = 0.75, gamma2 = 0.125, alpha1 = 6.0, beta1 = 3.0;
        double cnst = 1.0 / (alpha2 - beta1 * gamma2);
        double up1 = (alpha1 * alpha2 - beta1) * cnst;
        if (ibc % 2 != 0)
            for (long i = 0; i < N1; ++i) Av(i, 0) = (alpha2 * Av(i, 0) - beta1 * Av(i, 1)) * cnst;
        if (ibc == 1 || ibc == 2)
            for (long i = 0; i < N1; ++i) Av(i, N2 - 1) = (alpha2 * Av(i, N2 - 1) - beta1 * Av(i, N2 - 2)) * cnst;
        uppr[1] = (ibc % 2 == 0) ? 0.0 : up1;
        uppr[2] = alpha2;
        uppr[N2 - 1] = gamma2;
        for (int I = 1; I <= N2; ++I) lowr[I] = uppr[N2 - I + 1];
        lowr[N2] = (ibc != 1 && ibc != 2) ? 0.0 : up1;
        mtridag0(lowr.data() + 1, diag.data() + 1, uppr.data() + 1, A, N1, N2);
    } else {
        C1 = d2i * 7.0 / 9.0;
        C2 = d2i / 36.0;
        for (long J = 0; J < N1; ++J) {              // dbyd2.f90:212-220
            Av(J, 1) = C1 * (Bv(J, 2) - Bv(J, 0)) + C2 * (Bv(J, 3) - Bv(J, N2 - 1));
            Av(J, 0) = C1 * (Bv(J, 1) - Bv(J, N2 - 1)) + C2 * (Bv(J, 2) - Bv(J, N2 - 2));
            Av(J, N2 - 2) = C1 * (Bv(J, N2 - 1) - Bv(J, N2 - 3)) + C2 * (Bv(J, 0) - Bv(J, N2 - 4));
            Av(J, N2 - 1) = C1 * (Bv(J, 0) - Bv(J, N2 - 2)) + C2 * (Bv(J, 1) - Bv(J, N2 - 3));
        }
        double alpha = (double)(1.0f / 3.0f);
        for (int J = 1; J <= N2; ++J) { uppr[J] = alpha; lowr[J] = alpha; }
        mtridag1(lowr.data() + 1, diag.data() + 1, uppr.data() + 1, A, N1, N2);
    }
    return 0;
}

// ----------------------------------------------------------------------------
// Model state (initialize.f90 module globals that the path touches)
// ----------------------------------------------------------------------------
struct Model {
    oracle_params P;
    int nx, ny, nz, nzpml, dimfive, nf;
    long N;            // nx*ny*nz
    long NP;           // nx*ny
    double pi, rsun, normx, normy, dimc, dimrho, diml, dimb, deltat;
    double stretchx, stretchy, delta_width;
    int e_rad, o_rad, steps, freq_filtering, maxtime, forcing_length, cadforcing_step, num_steps;
    std::vector<double> x, y, z, stretch, unstretch, g, graw, gam1, source_dep, cq, rhoq;
    int npv = 2;       // PML auxiliary fields: 2 (quiet), 6 (MHD displacement form)
    // MHD background (option 10): B0, its curl as the reference forms it, the
    // horizontal background gradients, the sponge, the per-pixel source planes
    std::vector<double> box, boy, boz, curlbox, curlboy, curlboz, gradrho0_x, gradrho0_y, gradp0_x, gradp0_y;
    std::vector<double> spongez, spongexyz, delta_width_2d;
    std::vector<int> erad_2d, orad_2d;
    std::vector<cplx> eyekx, eyeky;
    std::vector<double> decay_coeff_x, decay_coeff_y;
    // 3-D background (quiet Sun still carries full arrays, as the reference does)
    std::vector<double> c2, rho0, p0, c_speed, rhoinv, c2rho0, gradrho0_z, gradp0_z, az, bzpml;
    std::vector<double> damping_rates;  // (nx/2+1, ny)
    // state
    std::vector<double> a, temp_step, scr, scrpml, pmlvars, psipml;
    std::vector<double> gradp, dvxdx, dvydy, gradvz, div, scratch;
    std::vector<double> forcing;   // (nx, ny)
    double betas[5];
    int time;
    // sources: planes (nx,ny,L) and mode
    int src_mode;  // 0 none, 1 forward series (plane 0 x series[n]), 2 lagrange over planes
    std::vector<double> vr;       // (nx, ny, L + 8), zero beyond L
    int vr_len;
    std::vector<double> series;   // forward time series, indexed by time (0-based)
    // kernels
    std::vector<double> kernelc2, kernelrho, hessian;
    // kernel mode of the 2-D MHD form (kernels.f90:99-133): B from the vector
    // potential as PRODUCE_KERNELS forms it, curl B0, and the B-field kernel
    std::vector<double> kbox, kboz, kcurlbox, kcurlboy, kcurlboz, kernelb;   // kernelb: (x, y, z) x N
    double* F(int l) { return &a[(long)l * N]; }
};

static inline long IDX(const Model& m, int i, int j, int k) { return i + (long)m.nx * (j + (long)m.ny * k); }

// ddz (derivatives.f90:10-24)
static void ddz(Model& m, const double* var, double* dvar, int bc) {
    oracle_dbyd2(dvar, var, m.NP, m.nz, bc);
#pragma omp parallel for schedule(static)
    for (int k = 0; k < m.nz; ++k)
        for (long ij = 0; ij < m.NP; ++ij) dvar[ij + m.NP * k] *= m.stretch[k];
}

// ddx (derivatives.f90:28-58): FFTW r2c along x, times eyekx, c2r, times stretchx
static void ddx(Model& m, const double* var, double* dvar) {
    int nx = m.nx;
#pragma omp parallel
    {
        std::vector<cplx> spec(nx / 2 + 1), work;
#pragma omp for schedule(static)
        for (long row = 0; row < (long)m.ny * m.nz; ++row) {
            r2c(var + row * nx, 1, nx, spec.data(), work);
            for (int i = 0; i < nx / 2 + 1; ++i) spec[i] = spec[i] * m.eyekx[i];
            c2r(spec.data(), nx, dvar + row * nx, 1, work);
        }
    }
    for (long q = 0; q < m.N; ++q) dvar[q] = dvar[q] * m.stretchx;
}

// ddy (derivatives.f90:62-170): transpose, r2c along y, times eyeky, c2r, times stretchy
static void ddy(Model& m, const double* var, double* dvar) {
    int nx = m.nx, ny = m.ny;
#pragma omp parallel
    {
        std::vector<cplx> spec(ny / 2 + 1), work;
        std::vector<double> col(ny), dcol(ny);
#pragma omp for schedule(static)
        for (long ik = 0; ik < (long)nx * m.nz; ++ik) {
            long i = ik % nx, k = ik / nx;
            for (int j = 0; j < ny; ++j) col[j] = var[IDX(m, i, j, k)];
            r2c(col.data(), 1, ny, spec.data(), work);
            for (int jj = 0; jj < ny / 2 + 1; ++jj) spec[jj] = spec[jj] * m.eyeky[jj];
            c2r(spec.data(), ny, dcol.data(), 1, work);
            for (int j = 0; j < ny; ++j) dvar[IDX(m, i, j, k)] = dcol[j];
        }
    }
    for (long q = 0; q < m.N; ++q) dvar[q] = dvar[q] * m.stretchy;
}

// ddxyz (derivatives.f90:175-305); the MPI overlap has no numerical effect
static void ddxyz(Model& m, const double* v1, double* d1, const double* v2, double* d2,
                  const double* v3, double* d3, int bc) {
    ddx(m, v1, d1);
    ddy(m, v2, d2);
    ddz(m, v3, d3, bc);
}

// 2-D FFTW r2c / c2r over the (x,y) plane, unnormalised (damping.f90:46-58)
static void plane_r2c(const Model& m, const double* in, cplx* out /* (nx/2+1, ny) */) {
    int nx = m.nx, ny = m.ny, h = nx / 2 + 1;
    std::vector<cplx> work, col(ny);
    for (int j = 0; j < ny; ++j) r2c(in + (long)j * nx, 1, nx, out + (long)j * h, work);
    for (int i = 0; i < h; ++i) {
        for (int j = 0; j < ny; ++j) col[j] = out[i + (long)j * h];
        fft_inplace(col.data(), ny, -1);
        for (int j = 0; j < ny; ++j) out[i + (long)j * h] = col[j];
    }
}
static void plane_c2r(const Model& m, const cplx* in, double* out) {
    int nx = m.nx, ny = m.ny, h = nx / 2 + 1;
    std::vector<cplx> tmp((long)h * ny), work, col(ny);
    for (int i = 0; i < h; ++i) {
        for (int j = 0; j < ny; ++j) col[j] = in[i + (long)j * h];
        fft_inplace(col.data(), ny, +1);
        for (int j = 0; j < ny; ++j) tmp[i + (long)j * h] = col[j];
    }
    for (int j = 0; j < ny; ++j) c2r(tmp.data() + (long)j * h, nx, out + (long)j * nx, 1, work);
}

// damp_velocity, 3-D branch (damping.f90:132-161)
static void damp_velocity(Model& m, const double* v, double* rhsv) {
    int h = m.nx / 2 + 1;
#pragma omp parallel
    {
        std::vector<cplx> spec((long)h * m.ny);
        std::vector<double> term(m.NP);
#pragma omp for schedule(static)
        for (int k = 0; k < m.nz; ++k) {
            plane_r2c(m, v + m.NP * k, spec.data());
            for (long q = 0; q < (long)h * m.ny; ++q) spec[q] = spec[q] * m.damping_rates[q];
            plane_c2r(m, spec.data(), term.data());
            for (long q = 0; q < m.NP; ++q) rhsv[q + m.NP * k] = rhsv[q + m.NP * k] - term[q];
        }
    }
}

// ----------------------------------------------------------------------------
// set-up
// ----------------------------------------------------------------------------
static void setup(Model& m, const oracle_params* P, const double* table /* (nz,6) row-major */) {
    m.P = *P;
    m.nx = P->nx; m.ny = P->ny; m.nz = P->nz;
    m.NP = (long)m.nx * m.ny; m.N = m.NP * m.nz;
    m.nzpml = P->npmlbot + P->npmltop;
    // velocity / MHD velocity / displacement form (initialize.f90:310-312)
    m.dimfive = P->option == 2 ? 5 : (P->option == 8 ? 8 : 6);
    m.nf = std::max(m.dimfive, 6);                   // fields held per state (a, temp_step, scr)
    m.pi = R4(3.14159265358979);                     // initialize.f90:38 (REAL*4 literal)
    m.rsun = R4(69598946770.0);
    m.normx = 1.0 / (double)m.nx; m.normy = 1.0 / (double)m.ny;
    int nx = m.nx, ny = m.ny, nz = m.nz;
    // grids (initialize.f90:192-212)
    m.x.resize(nx); m.y.resize(ny);
    for (int i = 0; i < nx; ++i) m.x[i] = (double)i / (double)nx;
    for (int j = 0; j < ny; ++j) m.y[j] = (double)j / (double)ny;
    m.eyekx.resize(nx / 2 + 1); m.eyeky.resize(ny / 2 + 1);
    for (int i = 0; i < nx / 2 + 1; ++i) m.eyekx[i] = cplx(0.0, (double)i) * m.normx * 2.0 * m.pi;
    for (int i = 0; i < ny / 2 + 1; ++i) m.eyeky[i] = cplx(0.0, (double)i) * m.normy * 2.0 * m.pi;
    // decay coefficients, evaluated in REAL*4 then scaled by normx (initialize.f90:215-221)
    m.decay_coeff_x.resize(nx / 2 + 1); m.decay_coeff_y.resize(ny / 2 + 1);
    for (int i = 1; i <= nx / 2 + 1; ++i) {
        float t = ((float)i - (float)nx / 3.0f) * 1.0f;
        float d = 1.0f / (1.0f + std::exp(t));
        m.decay_coeff_x[i - 1] = (double)d * m.normx;
    }
    for (int i = 1; i <= ny / 2 + 1; ++i) {
        float t = ((float)i - (float)ny / 3.0f) * 1.0f;
        float d = 1.0f / (1.0f + std::exp(t));
        m.decay_coeff_y[i - 1] = (double)d * m.normy;
    }
    m.stretchx = m.rsun / R4(P->xlength);
    m.stretchy = m.rsun / R4(P->ylength);
    // solar_data (initialize.f90:728-774)
    m.dimc = R4(1.0e6);
    m.dimrho = (double)1.0e-3f;
    m.diml = m.rsun;
    m.dimb = std::sqrt(4.0 * m.pi * m.dimc * m.dimc * m.dimrho);
    long N = m.N, NP = m.NP;
    m.z.resize(nz); m.g.resize(nz); m.graw.resize(nz); m.gam1.resize(nz); m.cq.resize(nz); m.rhoq.resize(nz);
    m.c2.assign(N, 0); m.rho0.assign(N, 0); m.p0.assign(N, 0); m.c_speed.assign(N, 0);
    for (int k = 0; k < nz; ++k) {
        const double* d = table + 6 * k;
        m.z[k] = d[0];
        double cs = d[1] / m.dimc;
        double c2v = (d[1] / m.dimc) * (d[1] / m.dimc);
        double r0 = d[2] / m.dimrho;
        double pp = d[3] / (m.dimrho * (m.dimc * m.dimc));
        for (long q = 0; q < NP; ++q) {
            m.c_speed[q + NP * k] = cs; m.c2[q + NP * k] = c2v;
            m.rho0[q + NP * k] = r0; m.p0[q + NP * k] = pp;
        }
        m.g[k] = d[4] * m.diml / (m.dimc * m.dimc);
        m.graw[k] = m.g[k];
        m.gam1[k] = d[5];
        m.cq[k] = d[1] / m.dimc;
        m.rhoq[k] = d[2] / m.dimrho;
    }
    // stretch (initialize.f90:464-468)
    m.unstretch.assign(nz, 0.0); m.stretch.assign(nz, 0.0);
    oracle_dbyd2(m.unstretch.data(), m.z.data(), 1, nz, 1);
    for (int k = 0; k < nz; ++k) m.stretch[k] = 1.0 / m.unstretch[k];
    m.deltat = P->timestep * m.dimc / m.diml;        // initialize.f90:472
    // READ_PARAMETERS (initialize.f90:978-981)
    double ts = R4(P->timestep), cad = R4(P->cadforcing);
    m.cadforcing_step = (int)std::floor(cad / ts);
    double nupeak = R4(P->nupeak);
    m.maxtime = (int)std::floor((R4(P->solartime) * 3600.0 + 2.0 / nupeak) / ts) + 2;
    m.maxtime = m.cadforcing_step * (int)std::floor((double)(m.maxtime / m.cadforcing_step) * 1.0);
    m.forcing_length = (int)std::floor((double)(m.maxtime / m.cadforcing_step) * 1.0) + 1;
    // driver.f90:269-281
    m.steps = (int)std::floor(R4(P->outputcad) / ts);
    m.freq_filtering = (int)std::floor(60.0 / ts);
    m.num_steps = (int)std::floor((double)m.maxtime * ts / cad) + 2;
    m.num_steps = 2 * (m.num_steps / 2) + 2;

    // ---------------- mp_Initialize_RHS (physics.f90:34-404) / _2d ----------------
    bool two_d = (P->option == 17 || P->option == 18);
    {
        double temp2 = 1.0 + R4(P->excitdep) / m.rsun, temp = 1.0;
        for (int k = 0; k < nz; ++k)
            if (std::fabs(m.z[k] - temp2) <= temp) { temp = std::fabs(m.z[k] - temp2); m.e_rad = k + 1; }
        double temp_r = 1.0 + R4(P->obsheight) / m.rsun; temp = 1.0;
        for (int k = 0; k < nz; ++k)
            if (std::fabs(m.z[k] - temp_r) <= temp) { temp = std::fabs(m.z[k] - temp_r); m.o_rad = k + 1; }
        if (two_d) { m.e_rad = nz - 5; m.o_rad = nz - 1; }   // physics2d.f90:42,54
    }
    if (P->compute_adjoint) m.delta_width = 2.0 / (m.z[m.o_rad] - m.z[m.o_rad - 2]);
    if (P->compute_forward) m.delta_width = 2.0 / (m.z[m.e_rad] - m.z[m.e_rad - 2]);
    m.source_dep.resize(nz);
    for (int k = 0; k < nz; ++k) {
        double dz = m.z[k] - m.z[m.e_rad - 1];
        m.source_dep[k] = std::exp(-R4(1.0e7) * 4.0 * (dz * dz));
    }
    m.rhoinv.resize(N); m.c2rho0.resize(N);
    for (long q = 0; q < N; ++q) { m.rhoinv[q] = 1.0 / m.rho0[q]; m.c2rho0[q] = m.c2[q] * m.rho0[q]; }
    m.gradrho0_z.assign(N, 0); m.gradp0_z.assign(N, 0);
    ddz(m, m.rho0.data(), m.gradrho0_z.data(), 1);
    ddz(m, m.p0.data(), m.gradp0_z.data(), 1);
    // PML profiles (physics.f90:255-303; physics2d.f90:293-342)
    m.az.assign(N, 0); m.bzpml.assign(N, 0);
    {
        int nb = P->npmlbot, nt = P->npmltop;
        double pml_a = m.pi * R4(0.005) * m.diml / m.dimc;
        double fac_bot = two_d ? 3.0 * 3.0 : 2.0 * 3.0 * 3.0;
        for (int k = 1; k <= nz; ++k) {
            double alphaz = pml_a;
            for (long q = 0; q < NP; ++q) {
                long id = q + NP * (k - 1);
                double dampz = 0.0, fdec = 1.0;
                if (k < nb + 1) {
                    alphaz = m.pi * R4(0.005) * m.diml / m.dimc * (m.z[k - 1] - m.z[0]) / (m.z[nb - 1] - m.z[0]);
                    double tempin = std::sqrt(m.c2[q]);          // tempin(:,:,1)
                    double r = (m.z[nb - 1] - m.z[k - 1]) / (m.z[nb - 1] - m.z[0]);
                    dampz = fac_bot * tempin / (m.z[nb - 1] - m.z[0]) * (r * r);
                    fdec = alphaz / (dampz + alphaz);
                    m.gradp0_z[id] = m.gradp0_z[id] * fdec;
                    m.gradrho0_z[id] = m.gradrho0_z[id] * fdec;
                }
                if (k > nz - nt) {
                    alphaz = m.pi * R4(0.005) * m.diml / m.dimc * (m.z[nz - 1] - m.z[k - 1]) / (m.z[nz - 1] - m.z[nz - nt]);
                    long qtop = two_d ? q + NP * (long)(nz - 6) : q + NP * (long)(nz - 1);  // tempin(:,:,nz-5) in 2-D
                    double tempin = std::sqrt(m.c2[qtop]);
                    double r = (m.z[nz - nt] - m.z[k - 1]) / (m.z[nz - 1] - m.z[nz - nt]);
                    dampz = 3.0 * 3.0 * tempin / (m.z[nz - 1] - m.z[nz - nt]) * (r * r);
                    fdec = alphaz / (dampz + alphaz);
                    m.gradp0_z[id] = m.gradp0_z[id] * fdec;
                    m.gradrho0_z[id] = m.gradrho0_z[id] * fdec;
                }
                if (q == 0 && (k < nb + 1 || k > nz - nt)) m.g[k - 1] = m.g[k - 1] * fdec;  // g(k)*functiondecay(1,1,k)
                m.bzpml[id] = -alphaz - dampz;
                m.az[id] = -dampz;
            }
        }
    }
    // INIT_DAMPING (damping.f90:10-65; 2-D variant :71-120)
    {
        int h = nx / 2 + 1;
        m.damping_rates.assign((long)h * ny, 0.0);
        double constx = 2.0 * m.pi / R4(P->xlength) * m.rsun;
        double consty = 2.0 * m.pi / R4(P->ylength) * m.rsun;
        double kayref = 902.0;
        double expo = (double)2.2f;
        double six = (double)1.0e-6f;
        for (int j = 1; j <= ny; ++j) {
            double jj;
            if (two_d) { if (j > 1) continue; jj = 0.0; }
            else jj = (j <= ny / 2 + 1) ? (double)(j - 1) : (double)(ny - j + 1);
            for (int i = 1; i <= h; ++i) {
                double ii = (double)(i - 1);
                double kay = std::sqrt(constx * constx * (ii * ii) + consty * consty * (jj * jj));
                m.damping_rates[(i - 1) + (long)h * (j - 1)] =
                    m.diml / m.dimc * six * 150.0 * std::pow(kay / kayref, expo) * m.normx * m.normy;
            }
        }
    }
    // INITIALIZE_STEP (step.f90:24-41), REAL*4 optimals
    {
        double opt[6];
        opt[1] = 1.0; opt[2] = 0.5;
        opt[3] = R4(0.1665579725791151184);
        opt[4] = R4(0.03950410250586729987);
        opt[5] = R4(0.007810706393337838236);
        double b[6];
        b[5] = opt[2];
        b[4] = opt[3] / b[5];
        b[3] = opt[4] / (b[5] * b[4]);
        b[2] = opt[5] / (b[5] * b[4] * b[3]);
        b[1] = 0.0;
        for (int i = 0; i < 5; ++i) m.betas[i] = b[i + 1] * m.deltat;
    }
    // state
    m.a.assign(N * m.nf, 0); m.temp_step.assign(N * m.nf, 0); m.scr.assign(N * m.nf, 0);
    m.npv = (P->option == 8 || P->option == 10 || P->option == 18) ? 6 : 2;
    long npml = (long)NP * std::max(m.nzpml, 1) * m.npv;
    m.scrpml.assign(npml, 0); m.pmlvars.assign(npml, 0); m.psipml.assign(npml, 0);
    m.gradp.assign(N * 3, 0); m.dvxdx.assign(N, 0); m.dvydy.assign(N, 0); m.gradvz.assign(N, 0);
    m.div.assign(N, 0); m.scratch.assign(N * 2, 0);
    m.forcing.assign(NP, 0);
    m.time = 0;
    m.src_mode = 0; m.vr_len = 0;
}

// ----------------------------------------------------------------------------
// MP_QUIET_PML_3D_DISPL (displacement.f90:482-658), option 4
// ----------------------------------------------------------------------------
static void rhs_option4(Model& m) {
    long N = m.N, NP = m.NP; int nz = m.nz;
    double* xi_x = &m.temp_step[0];
    double* xi_y = &m.temp_step[N];
    double* xi_z = &m.temp_step[2 * N];
    double* v_x = &m.temp_step[3 * N];
    double* v_y = &m.temp_step[4 * N];
    double* v_z = &m.temp_step[5 * N];
    double* RHSxi_x = &m.scr[0]; double* RHSxi_y = &m.scr[N]; double* RHSxi_z = &m.scr[2 * N];
    double* RHSv_x = &m.scr[3 * N]; double* RHSv_y = &m.scr[4 * N]; double* RHSv_z = &m.scr[5 * N];
    double* dxixdx = m.dvxdx.data(); double* dxiydy = m.dvydy.data(); double* dxizdz = m.gradvz.data();
    double* p = &m.scratch[N]; double* rho = &m.scratch[0];
    double* gradp_x = &m.gradp[0]; double* gradp_y = &m.gradp[N]; double* gradp_z = &m.gradp[2 * N];
    long PS = NP * m.nzpml;
    double* psivz = &m.psipml[0]; double* psip = &m.psipml[PS];
    double* RHSpsivz = &m.scrpml[0]; double* RHSpsip = &m.scrpml[PS];
    int nb = m.P.npmlbot, nt = m.P.npmltop;

    ddxyz(m, xi_x, dxixdx, xi_y, dxiydy, xi_z, dxizdz, 1);
    int pmlindex = 0;
    for (int k = 1; k <= nz; ++k) {
        if (k <= nb || k >= nz - nt + 1) {
            pmlindex++;
            for (long q = 0; q < NP; ++q) {
                long id = q + NP * (k - 1), ip = q + NP * (pmlindex - 1);
                RHSpsivz[ip] = m.az[id] * dxizdz[id] + m.bzpml[id] * psivz[ip];
                dxizdz[id] = dxizdz[id] + psivz[ip];
            }
        }
    }
#pragma omp parallel for schedule(static)
    for (long q = 0; q < N; ++q) {
        m.div[q] = dxixdx[q] + dxiydy[q] + dxizdz[q];
        p[q] = -m.c2rho0[q] * m.div[q] - xi_z[q] * m.gradp0_z[q];
        rho[q] = -m.rho0[q] * m.div[q] - xi_z[q] * m.gradrho0_z[q];
    }
    ddxyz(m, p, gradp_x, p, gradp_y, p, gradp_z, 0);
    pmlindex = 0;
    for (int k = 1; k <= nz; ++k) {
        if (k <= nb || k >= nz - nt + 1) {
            pmlindex++;
            for (long q = 0; q < NP; ++q) {
                long id = q + NP * (k - 1), ip = q + NP * (pmlindex - 1);
                RHSpsip[ip] = m.az[id] * gradp_z[id] + m.bzpml[id] * psip[ip];
                gradp_z[id] = gradp_z[id] + psip[ip];
            }
        }
    }
#pragma omp parallel for schedule(static)
    for (long q = 0; q < N; ++q) {
        RHSv_x[q] = -m.rhoinv[q] * gradp_x[q];
        RHSv_y[q] = -m.rhoinv[q] * gradp_y[q];
        RHSv_z[q] = -m.rhoinv[q] * gradp_z[q];
    }
    for (int k = 0; k < nz; ++k)
        for (long q = 0; q < NP; ++q) {
            long id = q + NP * k;
            RHSv_z[id] = RHSv_z[id] - rho[id] * m.g[k] * m.rhoinv[id];
        }
    for (long q = 0; q < N; ++q) { RHSxi_x[q] = v_x[q]; RHSxi_y[q] = v_y[q]; RHSxi_z[q] = v_z[q]; }
    // kernel-mode source (displacement.f90:609-634): plane o_rad (adjoint) / e_rad (forward)
    int ks = m.P.src_k > 0 ? m.P.src_k : (m.P.compute_adjoint ? m.o_rad : m.e_rad);
    if (m.src_mode != 0) {
        for (long q = 0; q < NP; ++q) {
            long id = q + NP * (ks - 1);
            RHSv_z[id] = RHSv_z[id] + m.forcing[q] / m.rho0[id] * m.delta_width;
        }
    }
    if (m.P.damp_waves) {
        damp_velocity(m, v_x, RHSv_x);
        damp_velocity(m, v_y, RHSv_y);
        damp_velocity(m, v_z, RHSv_z);
    }
    for (int l = 0; l < m.dimfive; ++l)
        for (long q = 0; q < NP; ++q) {
            m.scr[l * N + q + NP * (nz - 1)] = 0.0;
            m.scr[l * N + q] = 0.0;
        }
}

// ----------------------------------------------------------------------------
// MP_QUIET_PML_3D (pml.f90:12-76), option 2: velocity form, fields rho, v_x,
// v_y, v_z, p (initialize.f90:498-508); PML_BOUNDARY_ACCOUNTING_3D
// (pml.f90:213-231) for psi_vz and psi_p
// ----------------------------------------------------------------------------
static void rhs_option2(Model& m) {
    long N = m.N, NP = m.NP; int nz = m.nz;
    double* rho = &m.temp_step[0];
    double* v_x = &m.temp_step[N];
    double* v_y = &m.temp_step[2 * N];
    double* v_z = &m.temp_step[3 * N];
    double* p = &m.temp_step[4 * N];
    double* RHScont = &m.scr[0]; double* RHSv_x = &m.scr[N]; double* RHSv_y = &m.scr[2 * N];
    double* RHSv_z = &m.scr[3 * N]; double* RHSp = &m.scr[4 * N];
    double* dvxdx = m.dvxdx.data(); double* dvydy = m.dvydy.data(); double* dvzdz = m.gradvz.data();
    double* gradp_x = &m.gradp[0]; double* gradp_y = &m.gradp[N]; double* gradp_z = &m.gradp[2 * N];
    long PS = NP * m.nzpml;
    double* psivz = &m.psipml[0]; double* psip = &m.psipml[PS];
    double* RHSpsivz = &m.scrpml[0]; double* RHSpsip = &m.scrpml[PS];
    int nb = m.P.npmlbot, nt = m.P.npmltop;

    ddxyz(m, v_x, dvxdx, v_y, dvydy, v_z, dvzdz, 1);
    ddxyz(m, p, gradp_x, p, gradp_y, p, gradp_z, 0);
    int pmlindex = 0;
    for (int k = 1; k <= nz; ++k) {
        if (k <= nb || k >= nz - nt + 1) {
            pmlindex++;
            for (long q = 0; q < NP; ++q) {
                long id = q + NP * (k - 1), ip = q + NP * (pmlindex - 1);
                RHSpsip[ip] = m.az[id] * gradp_z[id] + m.bzpml[id] * psip[ip];
                gradp_z[id] = gradp_z[id] + psip[ip];
                RHSpsivz[ip] = m.az[id] * dvzdz[id] + m.bzpml[id] * psivz[ip];
                dvzdz[id] = dvzdz[id] + psivz[ip];
            }
        }
    }
#pragma omp parallel for schedule(static)
    for (long q = 0; q < N; ++q) {
        m.div[q] = dvxdx[q] + dvydy[q] + dvzdz[q];
        RHScont[q] = -m.gradrho0_z[q] * v_z[q] - m.rho0[q] * m.div[q];
        RHSv_x[q] = -m.rhoinv[q] * gradp_x[q];
        RHSv_y[q] = -m.rhoinv[q] * gradp_y[q];
    }
    int kc = m.P.src_k > 0 ? m.P.src_k : m.e_rad;
    for (int k = 1; k <= nz; ++k)
        for (long q = 0; q < NP; ++q) {
            long id = q + NP * (k - 1);
            RHSv_z[id] = -m.rhoinv[id] * (gradp_z[id] + rho[id] * m.g[k - 1]);
            if (std::abs(k - kc) <= 4 && m.src_mode != 0)
                RHSv_z[id] = RHSv_z[id] + m.forcing[q] * m.source_dep[k - 1];
        }
#pragma omp parallel for schedule(static)
    for (long q = 0; q < N; ++q) RHSp[q] = -m.c2rho0[q] * m.div[q] - v_z[q] * m.gradp0_z[q];
    for (int l = 0; l < 5; ++l)
        for (long q = 0; q < NP; ++q) {
            m.scr[l * N + q] = 0.0;
            m.scr[l * N + q + NP * (nz - 1)] = 0.0;
        }
    if (m.P.damp_waves) {
        damp_velocity(m, v_x, RHSv_x);
        damp_velocity(m, v_y, RHSv_y);
        damp_velocity(m, v_z, RHSv_z);
    }
}

// ----------------------------------------------------------------------------
// MHD background (option 10): the magnetic parts of mp_Initialize_RHS
// (physics.f90:62-161, 204-208, 255-303, 356-363) in the reference's order,
// applied after the quiet set-up.  Inputs are the 3-D cgs arrays that
// READ_IN_FIELD reads (all_modules.f90:486-513), (nz, ny, nx) C order.
// ----------------------------------------------------------------------------
static void setup_mhd(Model& m, const double* rho, const double* cs, const double* pr,
                      const double* bx, const double* by, const double* bz) {
    long N = m.N, NP = m.NP; int nx = m.nx, ny = m.ny, nz = m.nz;
    // erad_2d / orad_2d (physics.f90:62-87): the search runs before
    // READ_IN_FIELD, on the density of solar_data (the quiet column); the
    // loop bounds are clamped to the box
    m.erad_2d.assign(NP, 0); m.orad_2d.assign(NP, 0); m.delta_width_2d.assign(NP, 0.0);
    for (long q = 0; q < NP; ++q) {
        double temp = 1.0;
        for (int k = std::max(1, m.e_rad - 50); k <= std::min(nz, m.e_rad + 10); ++k)
            if (std::fabs(m.rhoq[m.e_rad - 1] - m.rho0[q + NP * (k - 1)]) <= temp) {
                temp = std::fabs(m.rhoq[m.e_rad - 1] - m.rho0[q + NP * (k - 1)]);
                m.erad_2d[q] = k;
            }
        temp = 1.0;
        for (int k = std::max(1, m.o_rad - 50); k <= std::min(nz, m.o_rad + 10); ++k)
            if (std::fabs(m.rhoq[m.o_rad - 1] - m.rho0[q + NP * (k - 1)]) <= temp) {
                temp = std::fabs(m.rhoq[m.o_rad - 1] - m.rho0[q + NP * (k - 1)]);
                m.orad_2d[q] = k;
            }
        const int k2 = m.P.compute_adjoint ? m.orad_2d[q] : m.erad_2d[q];
        m.delta_width_2d[q] = 2.0 / (m.z[k2] - m.z[k2 - 2]);
    }
    // spongez (physics.f90:104-108); PERIODIC: spongexyz(:,:,k) = spongez(k)
    m.spongez.assign(nz, 0.0); m.spongexyz.assign(N, 0.0);
    for (int k = 0; k < nz; ++k) {
        m.spongez[k] = 200.0 / (1.0 + std::exp((R4(1.002) - m.z[k]) / R4(0.0001)))
                     + 300.0 / (1.0 + std::exp((m.z[k] - (m.z[0] + R4(0.005))) / R4(0.0005)));
        for (long q = 0; q < NP; ++q) m.spongexyz[q + NP * k] = m.spongez[k];
    }
    // READ_IN_FIELD
    m.box.assign(N, 0); m.boy.assign(N, 0); m.boz.assign(N, 0);
    for (long q = 0; q < N; ++q) {
        m.rho0[q] = rho[q] / m.dimrho;
        m.c_speed[q] = cs[q] / m.dimc;
        m.p0[q] = pr[q] / (m.dimrho * std::pow(m.dimc, 2.0));
        m.box[q] = bx[q] / m.dimb; m.boy[q] = by[q] / m.dimb; m.boz[q] = bz[q] / m.dimb;
        m.c2[q] = std::pow(m.c_speed[q], 2.0);
    }
    // reduction of the field (physics.f90:116-129): the top taper is REAL*4
    std::vector<double> red(N);
    for (int k = 0; k < nz; ++k)
        for (long q = 0; q < NP; ++q) {
            long id = q + NP * k;
            red[id] = (std::pow(m.boz[id], 2.0) + std::pow(m.box[id], 2.0) + std::pow(m.boy[id], 2.0))
                    / (m.rho0[id] * std::pow(m.cq[k], 2.0));
        }
    for (long q = 0; q < N; ++q) red[q] = 8.0 / (8.0 + red[q]);
    for (int k1 = nz - 10; k1 <= nz; ++k1) {
        if (k1 < 1) continue;
        const float t = (float)(k1 - nz) / 10.0f;
        const double f = (double)std::pow(t, 4.0f);
        for (long q = 0; q < NP; ++q) red[q + NP * (k1 - 1)] *= f;
    }
    for (long q = 0; q < N; ++q) {
        const double s = std::pow(red[q], 0.5);
        m.box[q] *= s; m.boy[q] *= s; m.boz[q] *= s;
    }
    // curl B0 as formed at physics.f90:131-159: the d/dz parts are discarded
    m.curlbox.assign(N, 0); m.curlboy.assign(N, 0); m.curlboz.assign(N, 0);
    ddx(m, m.boy.data(), m.curlboz.data());
    ddy(m, m.box.data(), red.data());
    for (long q = 0; q < N; ++q) m.curlboz[q] = m.curlboz[q] - red[q];
    ddy(m, m.boz.data(), m.curlbox.data());
    ddx(m, m.boz.data(), red.data());
    for (long q = 0; q < N; ++q) m.curlboy[q] = 0.0 - red[q];
    // physics.f90:204-208
    for (long q = 0; q < N; ++q) { m.rhoinv[q] = 1.0 / m.rho0[q]; m.c2rho0[q] = m.c2[q] * m.rho0[q]; }
    ddz(m, m.rho0.data(), m.gradrho0_z.data(), 1);
    ddz(m, m.p0.data(), m.gradp0_z.data(), 1);
    // PML profiles with the magnetic wave speed (physics.f90:255-303)
    {
        int nb = m.P.npmlbot, nt = m.P.npmltop;
        std::vector<double> tempin(N);
        for (long q = 0; q < N; ++q)
            tempin[q] = std::pow(m.c2[q] + (std::pow(m.box[q], 2.0) + std::pow(m.boy[q], 2.0)
                                            + std::pow(m.boz[q], 2.0)) / m.rho0[q], 0.5);
        for (int k = 1; k <= nz; ++k) {
            double alphaz = m.pi * R4(0.005) * m.diml / m.dimc;
            if (k < nb + 1) alphaz = m.pi * R4(0.005) * m.diml / m.dimc * (m.z[k - 1] - m.z[0]) / (m.z[nb - 1] - m.z[0]);
            if (k > nz - nt) alphaz = m.pi * R4(0.005) * m.diml / m.dimc * (m.z[nz - 1] - m.z[k - 1]) / (m.z[nz - 1] - m.z[nz - nt]);
            double fdec00 = 1.0;
            for (long q = 0; q < NP; ++q) {
                long id = q + NP * (k - 1);
                double dampz = 0.0, fdec = 1.0;
                if (k < nb + 1) {
                    double r = (m.z[nb - 1] - m.z[k - 1]) / (m.z[nb - 1] - m.z[0]);
                    dampz = 2.0 * 3.0 * 3.0 * tempin[q] / (m.z[nb - 1] - m.z[0]) * (r * r);
                    fdec = alphaz / (dampz + alphaz);
                    m.gradp0_z[id] *= fdec; m.gradrho0_z[id] *= fdec;
                }
                if (k > nz - nt) {
                    double r = (m.z[nz - nt] - m.z[k - 1]) / (m.z[nz - 1] - m.z[nz - nt]);
                    dampz = 3.0 * 3.0 * tempin[q + NP * (long)(nz - 1)] / (m.z[nz - 1] - m.z[nz - nt]) * (r * r);
                    fdec = alphaz / (dampz + alphaz);
                    m.gradp0_z[id] *= fdec; m.gradrho0_z[id] *= fdec;
                }
                if (q == 0) fdec00 = fdec;
                m.bzpml[id] = -alphaz - dampz;
                m.az[id] = -dampz;
            }
            m.g[k - 1] = (k < nb + 1 || k > nz - nt) ? m.graw[k - 1] * fdec00 : m.graw[k - 1];
        }
    }
    // horizontal background gradients (physics.f90:356-363)
    m.gradrho0_x.assign(N, 0); m.gradrho0_y.assign(N, 0); m.gradp0_x.assign(N, 0); m.gradp0_y.assign(N, 0);
    ddx(m, m.rho0.data(), m.gradrho0_x.data());
    ddy(m, m.rho0.data(), m.gradrho0_y.data());
    ddx(m, m.p0.data(), m.gradp0_x.data());
    ddy(m, m.p0.data(), m.gradp0_y.data());
    (void)nx; (void)ny;
}

static inline void cross3(double ax, double ay, double az, double bx, double by, double bz,
                          double& cx, double& cy, double& cz) {
    cx = ay * bz - az * by;
    cy = az * bx - ax * bz;
    cz = ax * by - ay * bx;
}

// ----------------------------------------------------------------------------
// MP_MHD_PML_3D (pml.f90:80-208), option 8: the MHD velocity form, fields
// rho, v_x, v_y, v_z, p, b_x, b_y, b_z (initialize.f90:498-510, 545-551);
// PML_BOUNDARY_ACCOUNTING_3D (pml.f90:213-285) at both ends with psi_p,
// psi_vz, psi_induction_bx (on d flux2/dz), psi_induction_by (on d flux1/dz),
// psi_dzbx, psi_dzby; source forcing*source_dep(k) for |k - e_rad| <= 4
// ----------------------------------------------------------------------------
static void rhs_option8(Model& m) {
    long N = m.N, NP = m.NP; int nz = m.nz;
    double* rho = &m.temp_step[0];
    double* v_x = &m.temp_step[N]; double* v_y = &m.temp_step[2 * N]; double* v_z = &m.temp_step[3 * N];
    double* p = &m.temp_step[4 * N];
    double* bx = &m.temp_step[5 * N]; double* by = &m.temp_step[6 * N]; double* bz = &m.temp_step[7 * N];
    double* RHScont = &m.scr[0];
    double* RHSv_x = &m.scr[N]; double* RHSv_y = &m.scr[2 * N]; double* RHSv_z = &m.scr[3 * N];
    double* RHSp = &m.scr[4 * N];
    double* RHSb_x = &m.scr[5 * N]; double* RHSb_y = &m.scr[6 * N]; double* RHSb_z = &m.scr[7 * N];
    long PS = NP * m.nzpml;
    double* psivz = &m.psipml[0]; double* psip = &m.psipml[PS];
    double* psidzbx = &m.psipml[2 * PS]; double* psidzby = &m.psipml[3 * PS];
    double* psiibx = &m.psipml[4 * PS]; double* psiiby = &m.psipml[5 * PS];
    double* RHSpsivz = &m.scrpml[0]; double* RHSpsip = &m.scrpml[PS];
    double* RHSpsidzbx = &m.scrpml[2 * PS]; double* RHSpsidzby = &m.scrpml[3 * PS];
    double* RHSpsiibx = &m.scrpml[4 * PS]; double* RHSpsiiby = &m.scrpml[5 * PS];
    int nb = m.P.npmlbot, nt = m.P.npmltop;
    std::vector<double> flux1(N), flux2(N), flux3(N), dvxdx(N), dvydy(N), dvzdz(N);
    std::vector<double> gradp_x(N), gradp_y(N), gradp_z(N), dzflux1(N), dzflux2(N);
    std::vector<double> curlbx(N), curlby(N), curlbz(N), dzbx(N), dzby(N);
    for (long q = 0; q < N; ++q) {
        flux1[q] = -(v_z[q] * m.boy[q] - v_y[q] * m.boz[q]);
        flux2[q] = -(v_x[q] * m.boz[q] - v_z[q] * m.box[q]);
        flux3[q] = -(v_y[q] * m.box[q] - v_x[q] * m.boy[q]);
    }
    // the six ddxyz calls of pml.f90:106-116, in order (flux2 and flux3 are
    // reused as outputs once their derivatives are taken)
    ddxyz(m, v_x, dvxdx.data(), v_y, dvydy.data(), v_z, dvzdz.data(), 1);
    ddxyz(m, flux3.data(), RHSb_y, p, gradp_y.data(), flux1.data(), dzflux1.data(), 1);
    ddxyz(m, p, gradp_x.data(), flux3.data(), RHSb_x, flux2.data(), dzflux2.data(), 1);
    ddxyz(m, flux2.data(), RHSb_z, bz, curlbx.data(), bx, dzbx.data(), 1);
    ddxyz(m, by, curlbz.data(), bx, flux2.data(), p, gradp_z.data(), 1);
    ddxyz(m, bz, curlby.data(), flux1.data(), flux3.data(), by, dzby.data(), 1);
    // PML_BOUNDARY_ACCOUNTING_3D
    int pmlindex = 0;
    for (int k = 1; k <= nz; ++k) {
        if (k <= nb || k >= nz - nt + 1) {
            pmlindex++;
            for (long q = 0; q < NP; ++q) {
                long id = q + NP * (k - 1), ip = q + NP * (pmlindex - 1);
                RHSpsip[ip] = m.az[id] * gradp_z[id] + m.bzpml[id] * psip[ip];
                gradp_z[id] = gradp_z[id] + psip[ip];
                RHSpsivz[ip] = m.az[id] * dvzdz[id] + m.bzpml[id] * psivz[ip];
                dvzdz[id] = dvzdz[id] + psivz[ip];
            }
        }
    }
    pmlindex = 0;
    for (int k = 1; k <= nz; ++k) {
        if (k <= nb || k >= nz - nt + 1) {
            pmlindex++;
            for (long q = 0; q < NP; ++q) {
                long id = q + NP * (k - 1), ip = q + NP * (pmlindex - 1);
                RHSpsiibx[ip] = m.az[id] * dzflux2[id] + m.bzpml[id] * psiibx[ip];
                dzflux2[id] = dzflux2[id] + psiibx[ip];
                RHSpsiiby[ip] = m.az[id] * dzflux1[id] + m.bzpml[id] * psiiby[ip];
                dzflux1[id] = dzflux1[id] + psiiby[ip];
                RHSpsidzbx[ip] = m.az[id] * dzbx[id] + m.bzpml[id] * psidzbx[ip];
                dzbx[id] = dzbx[id] + psidzbx[ip];
                RHSpsidzby[ip] = m.az[id] * dzby[id] + m.bzpml[id] * psidzby[ip];
                dzby[id] = dzby[id] + psidzby[ip];
            }
        }
    }
    for (long q = 0; q < N; ++q) {
        RHSb_x[q] = RHSb_x[q] - dzflux2[q];
        RHSb_y[q] = -RHSb_y[q] + dzflux1[q];
        RHSb_z[q] = RHSb_z[q] - flux3[q];
        const double div = dvxdx[q] + dvydy[q] + dvzdz[q];
        curlbx[q] = curlbx[q] - dzby[q];
        curlby[q] = -curlby[q] + dzbx[q];
        curlbz[q] = curlbz[q] - flux2[q];
        RHScont[q] = -m.gradrho0_x[q] * v_x[q] - m.gradrho0_y[q] * v_y[q] - m.gradrho0_z[q] * v_z[q] - m.rho0[q] * div;
        RHSp[q] = -m.c2rho0[q] * div - v_x[q] * m.gradp0_x[q] - v_y[q] * m.gradp0_y[q] - v_z[q] * m.gradp0_z[q];
        double f1, f2, f3;
        cross3(curlbx[q], curlby[q], curlbz[q], m.box[q], m.boy[q], m.boz[q], f1, f2, f3);
        RHSv_x[q] = -m.rhoinv[q] * (gradp_x[q] - f1);
        RHSv_y[q] = -m.rhoinv[q] * (gradp_y[q] - f2);
        RHSv_z[q] = -m.rhoinv[q] * (gradp_z[q] - f3);
        cross3(m.curlbox[q], m.curlboy[q], m.curlboz[q], bx[q], by[q], bz[q], f1, f2, f3);
        RHSv_x[q] = RHSv_x[q] + m.rhoinv[q] * f1;
        RHSv_y[q] = RHSv_y[q] + m.rhoinv[q] * f2;
        RHSv_z[q] = RHSv_z[q] + m.rhoinv[q] * f3;
    }
    int kc = m.P.src_k > 0 ? m.P.src_k : m.e_rad;
    for (int k = 1; k <= nz; ++k)
        for (long q = 0; q < NP; ++q) {
            long id = q + NP * (k - 1);
            RHSv_z[id] = RHSv_z[id] - m.rhoinv[id] * rho[id] * m.g[k - 1];
            if (std::abs(k - kc) <= 4 && m.src_mode != 0)
                RHSv_z[id] = RHSv_z[id] + m.forcing[q] * m.source_dep[k - 1];
        }
    for (int l = 0; l < 8; ++l)
        for (long q = 0; q < NP; ++q) {
            m.scr[l * N + q + NP * (nz - 1)] = 0.0;
            m.scr[l * N + q] = 0.0;
        }
    if (m.P.damp_waves) {
        damp_velocity(m, v_x, RHSv_x);
        damp_velocity(m, v_y, RHSv_y);
        damp_velocity(m, v_z, RHSv_z);
    }
}

// ----------------------------------------------------------------------------
// MP_MHD_PML_3D_DISPL (displacement.f90:663-849), option 10: the PML sits at
// the bottom only (k <= npmlbot) with six auxiliaries: psi_vz, psi_p,
// psi_dzbx, psi_dzby, psi_induction_bx, psi_induction_by (initialize.f90:
// 487-490, 560-566); the top has the sponge over the last 36 planes
// ----------------------------------------------------------------------------
static void rhs_option10(Model& m) {
    long N = m.N, NP = m.NP; int nz = m.nz;
    double* xi_x = &m.temp_step[0]; double* xi_y = &m.temp_step[N]; double* xi_z = &m.temp_step[2 * N];
    double* v_x = &m.temp_step[3 * N]; double* v_y = &m.temp_step[4 * N]; double* v_z = &m.temp_step[5 * N];
    double* RHSxi_x = &m.scr[0]; double* RHSxi_y = &m.scr[N]; double* RHSxi_z = &m.scr[2 * N];
    double* RHSv_x = &m.scr[3 * N]; double* RHSv_y = &m.scr[4 * N]; double* RHSv_z = &m.scr[5 * N];
    long PS = NP * m.nzpml;
    double* psivz = &m.psipml[0]; double* psip = &m.psipml[PS];
    double* psidzbx = &m.psipml[2 * PS]; double* psidzby = &m.psipml[3 * PS];
    double* psiibx = &m.psipml[4 * PS]; double* psiiby = &m.psipml[5 * PS];
    double* RHSpsivz = &m.scrpml[0]; double* RHSpsip = &m.scrpml[PS];
    double* RHSpsidzbx = &m.scrpml[2 * PS]; double* RHSpsidzby = &m.scrpml[3 * PS];
    double* RHSpsiibx = &m.scrpml[4 * PS]; double* RHSpsiiby = &m.scrpml[5 * PS];
    int nb = m.P.npmlbot;
    std::vector<double> flux1(N), flux2(N), flux3(N), dxixdx(N), dxiydy(N), dxizdz(N), p(N), rho(N);
    std::vector<double> gradp_x(N), gradp_y(N), gradp_z(N), bxv(N), byv(N), bzv(N), dzflux1(N), dzflux2(N);
    std::vector<double> curlbx(N), curlby(N), curlbz(N), dzbx(N), dzby(N);
    for (long q = 0; q < N; ++q) {
        flux1[q] = -(xi_z[q] * m.boy[q] - xi_y[q] * m.boz[q]);
        flux2[q] = -(xi_x[q] * m.boz[q] - xi_z[q] * m.box[q]);
        flux3[q] = -(xi_y[q] * m.box[q] - xi_x[q] * m.boy[q]);
    }
    ddxyz(m, xi_x, dxixdx.data(), xi_y, dxiydy.data(), xi_z, dxizdz.data(), 1);
    auto pml_bottom = [&](double* deriv, double* psi, double* rhs) {
        for (int k = 1; k <= nb; ++k)
            for (long q = 0; q < NP; ++q) {
                long id = q + NP * (k - 1), ip = q + NP * (k - 1);
                rhs[ip] = m.az[id] * deriv[id] + m.bzpml[id] * psi[ip];
                deriv[id] = deriv[id] + psi[ip];
            }
    };
    pml_bottom(dxizdz.data(), psivz, RHSpsivz);
    for (long q = 0; q < N; ++q) {
        const double div = dxixdx[q] + dxiydy[q] + dxizdz[q];
        p[q] = -m.c2rho0[q] * div - xi_z[q] * m.gradp0_z[q] - xi_x[q] * m.gradp0_x[q] - xi_y[q] * m.gradp0_y[q];
        rho[q] = -m.rho0[q] * div - xi_z[q] * m.gradrho0_z[q] - xi_x[q] * m.gradrho0_x[q] - xi_y[q] * m.gradrho0_y[q];
    }
    ddxyz(m, p.data(), gradp_x.data(), p.data(), gradp_y.data(), p.data(), gradp_z.data(), 0);
    pml_bottom(gradp_z.data(), psip, RHSpsip);
    // induction: b = curl(xi x B0) from the fluxes (displacement.f90:716-757)
    ddx(m, flux3.data(), byv.data());
    ddy(m, flux3.data(), bxv.data());
    ddz(m, flux2.data(), dzflux2.data(), 1);
    ddx(m, flux2.data(), bzv.data());
    ddy(m, flux1.data(), flux3.data());
    ddz(m, flux1.data(), dzflux1.data(), 1);
    for (int k = 1; k <= nb; ++k)
        for (long q = 0; q < NP; ++q) {
            long id = q + NP * (k - 1), ip = id;
            RHSpsiibx[ip] = m.az[id] * dzflux2[id] + m.bzpml[id] * psiibx[ip];
            dzflux2[id] = dzflux2[id] + psiibx[ip];
            RHSpsiiby[ip] = m.az[id] * dzflux1[id] + m.bzpml[id] * psiiby[ip];
            dzflux1[id] = dzflux1[id] + psiiby[ip];
        }
    for (long q = 0; q < N; ++q) {
        bxv[q] = bxv[q] - dzflux2[q];
        byv[q] = -byv[q] + dzflux1[q];
        bzv[q] = bzv[q] - flux3[q];
    }
    // curl b (displacement.f90:759-787)
    ddx(m, byv.data(), curlbz.data());
    ddy(m, bzv.data(), curlbx.data());
    ddz(m, bxv.data(), dzbx.data(), 1);
    ddx(m, bzv.data(), curlby.data());
    ddy(m, bxv.data(), flux1.data());
    ddz(m, byv.data(), dzby.data(), 1);
    for (int k = 1; k <= nb; ++k)
        for (long q = 0; q < NP; ++q) {
            long id = q + NP * (k - 1), ip = id;
            RHSpsidzbx[ip] = m.az[id] * dzbx[id] + m.bzpml[id] * psidzbx[ip];
            dzbx[id] = dzbx[id] + psidzbx[ip];
            RHSpsidzby[ip] = m.az[id] * dzby[id] + m.bzpml[id] * psidzby[ip];
            dzby[id] = dzby[id] + psidzby[ip];
        }
    for (long q = 0; q < N; ++q) {
        curlbx[q] = curlbx[q] - dzby[q];
        curlby[q] = -curlby[q] + dzbx[q];
        curlbz[q] = curlbz[q] - flux1[q];
    }
    for (long q = 0; q < N; ++q) {
        double f1, f2, f3;
        cross3(curlbx[q], curlby[q], curlbz[q], m.box[q], m.boy[q], m.boz[q], f1, f2, f3);
        RHSv_x[q] = m.rhoinv[q] * (-gradp_x[q] + f1);
        RHSv_y[q] = m.rhoinv[q] * (-gradp_y[q] + f2);
        RHSv_z[q] = m.rhoinv[q] * (-gradp_z[q] + f3);
        cross3(m.curlbox[q], m.curlboy[q], m.curlboz[q], bxv[q], byv[q], bzv[q], f1, f2, f3);
        RHSv_x[q] = RHSv_x[q] + m.rhoinv[q] * f1;
        RHSv_y[q] = RHSv_y[q] + m.rhoinv[q] * f2;
        RHSv_z[q] = RHSv_z[q] + m.rhoinv[q] * f3;
    }
    for (int k = std::max(1, nz - 35); k <= nz; ++k)
        for (long q = 0; q < NP; ++q) {
            long id = q + NP * (k - 1);
            RHSv_x[id] = RHSv_x[id] - m.spongexyz[id] * v_x[id];
            RHSv_y[id] = RHSv_y[id] - m.spongexyz[id] * v_y[id];
            RHSv_z[id] = RHSv_z[id] - m.spongexyz[id] * v_z[id];
        }
    for (int k = 0; k < nz; ++k)
        for (long q = 0; q < NP; ++q) {
            long id = q + NP * k;
            RHSv_z[id] = RHSv_z[id] - m.rhoinv[id] * rho[id] * m.g[k];
        }
    for (long q = 0; q < N; ++q) { RHSxi_x[q] = v_x[q]; RHSxi_y[q] = v_y[q]; RHSxi_z[q] = v_z[q]; }
    if (m.P.damp_waves) {
        damp_velocity(m, v_x, RHSv_x);
        damp_velocity(m, v_y, RHSv_y);
        damp_velocity(m, v_z, RHSv_z);
    }
    // kernel-mode source on the per-pixel planes while time <= forcing_length*cadforcing_step
    if (m.src_mode != 0 && m.time <= m.forcing_length * m.cadforcing_step) {
        for (long q = 0; q < NP; ++q) {
            const int k2 = m.P.src_k > 0 ? m.P.src_k : (m.P.compute_adjoint ? m.orad_2d[q] : m.erad_2d[q]);
            long id = q + NP * (k2 - 1);
            RHSv_z[id] = RHSv_z[id] + m.forcing[q] / m.rho0[id] * m.delta_width_2d[q];
        }
    }
    for (int l = 0; l < 6; ++l)
        for (long q = 0; q < NP; ++q) {
            m.scr[l * N + q + NP * (nz - 1)] = 0.0;
            m.scr[l * N + q] = 0.0;
        }
}

// ----------------------------------------------------------------------------
// DBYD1 (dbyd1.f) for ibc = 0: the compact first derivative of DBYD2 along
// the first index, with the coefficients in default REAL (REAL*4) as that
// file declares none, the end rows zero, solved by TRIDAG (tridag.f, the
// Thomas algorithm with divisions).  a, b: (n2, n1) C order (n1 fastest).
// ----------------------------------------------------------------------------
static void dbyd1_ibc0(double* a, const double* b, int n1, long n2) {
    const float d1i = (float)(n1 - 1);
    const double C1 = (double)(d1i * 7.0f / 9.0f), C2 = (double)(d1i / 36.0f);
    const double B1 = (double)(-43.0f / 96.0f * d1i), B2 = (double)(-5.0f / 6.0f * d1i);
    const double B3 = (double)(9.0f / 8.0f * d1i), B4 = (double)(1.0f / 6.0f * d1i), B5 = (double)(-1.0f / 96.0f * d1i);
    std::vector<double> uppr(n1 + 1, 0.0), lowr(n1 + 1, 0.0), diag(n1 + 1, 1.0);
    for (int J = 3; J <= n1 - 2; ++J) uppr[J] = (double)(1.0f / 3.0f);
    uppr[1] = 0.0;                                  // mod(ibc,2) == 0
    uppr[2] = (double)(3.0f / 4.0f);
    uppr[n1 - 1] = (double)(1.0f / 8.0f);
    for (int I = 1; I <= n1; ++I) lowr[I] = uppr[n1 - I + 1];
    lowr[n1] = 0.0;                                 // ibc /= 1, 2
    std::vector<double> gam(n1 + 1), ud(n1 + 1), r(n1 + 1);
    for (long i = 0; i < n2; ++i) {
        const double* B = b + i * n1 - 1;           // 1-based
        double* A = a + i * n1 - 1;
        for (int J = 3; J <= n1 - 2; ++J) r[J] = C1 * (B[J + 1] - B[J - 1]) + C2 * (B[J + 2] - B[J - 2]);
        r[2] = B1 * B[1] + B2 * B[2] + B3 * B[3] + B4 * B[4] + B5 * B[5];
        r[n1 - 1] = -(B1 * B[n1] + B2 * B[n1 - 1] + B3 * B[n1 - 2] + B4 * B[n1 - 3] + B5 * B[n1 - 4]);
        r[1] = 0.0;
        r[n1] = 0.0;
        // TRIDAG(LOWR, DIAG, UPPR, A, A, N1, 0)
        double bet = diag[1];
        ud[1] = r[1] / bet;
        for (int J = 2; J <= n1; ++J) {
            gam[J] = uppr[J - 1] / bet;
            bet = diag[J] - lowr[J] * gam[J];
            ud[J] = (r[J] - lowr[J] * ud[J - 1]) / bet;
        }
        for (int J = n1 - 1; J >= 1; --J) ud[J] = ud[J] - gam[J + 1] * ud[J + 1];
        for (int J = 1; J <= n1; ++J) A[J] = ud[J];
    }
}

// ----------------------------------------------------------------------------
// 2-D MHD background (option 18, kernel mode): the magnetic part of
// mp_Initialize_RHS_2d (physics2d.f90:106-195) and the rest of it in order
// (:223-226 gradients, :262-297 PML with the magnetic wave speed, :318-341
// horizontal gradients and source planes).  Inputs (nz, nx) cgs: pressure,
// density, sound speed (model_c) and the vector potential psi
// (model_vectorpsi): B_x = -d psi/dz, B_z = DBYD1(psi) * stretchx.
// ----------------------------------------------------------------------------
static void setup_mhd2d(Model& m, const double* pr, const double* rho, const double* cs, const double* psi) {
    long N = m.N, NP = m.NP; int nx = m.nx, nz = m.nz;
    m.box.assign(N, 0); m.boy.assign(N, 0); m.boz.assign(N, 0);
    ddz(m, psi, m.box.data(), 1);
    for (long q = 0; q < N; ++q) m.box[q] = -m.box[q];
    dbyd1_ibc0(m.boz.data(), psi, nx, (long)nz);
    for (long q = 0; q < N; ++q) m.boz[q] = m.boz[q] * m.stretchx;
    for (long q = 0; q < N; ++q) {
        m.box[q] = m.box[q] / m.dimb;
        m.boz[q] = m.boz[q] / m.dimb;
        m.p0[q] = pr[q] / (m.dimrho * std::pow(m.dimc, 2.0));
        m.rho0[q] = rho[q] / m.dimrho;
        m.c_speed[q] = cs[q] / m.dimc;
        m.c2[q] = std::pow(m.c_speed[q], 2.0);
    }
    for (int k = 0; k < nz; ++k) { m.cq[k] = m.c_speed[NP * k]; m.rhoq[k] = m.rho0[NP * k]; }
    // curl B0 (physics2d.f90:180-183; the reduction is computed, then reset to 1)
    std::vector<double> tmp(N);
    m.curlbox.assign(N, 0); m.curlboy.assign(N, 0); m.curlboz.assign(N, 0);
    ddz(m, m.box.data(), m.curlboy.data(), 1);
    ddx(m, m.boz.data(), tmp.data());
    for (long q = 0; q < N; ++q) m.curlboy[q] = m.curlboy[q] - tmp[q];
    // physics2d.f90:223-226
    for (long q = 0; q < N; ++q) { m.rhoinv[q] = 1.0 / m.rho0[q]; m.c2rho0[q] = m.c2[q] * m.rho0[q]; }
    ddz(m, m.rho0.data(), m.gradrho0_z.data(), 1);
    ddz(m, m.p0.data(), m.gradp0_z.data(), 1);
    // PML (physics2d.f90:262-297): tempin at k = 1 (bottom) and nz-5 (top), factor 3*3 at both ends
    {
        int nb = m.P.npmlbot, nt = m.P.npmltop;
        std::vector<double> tempin(N);
        for (long q = 0; q < N; ++q)
            tempin[q] = std::pow(m.c2[q] + (std::pow(m.box[q], 2.0) + std::pow(m.boz[q], 2.0)) / m.rho0[q], 0.5);
        for (int k = 1; k <= nz; ++k) {
            double alphaz = m.pi * R4(0.005) * m.diml / m.dimc;
            if (k < nb + 1) alphaz = m.pi * R4(0.005) * m.diml / m.dimc * (m.z[k - 1] - m.z[0]) / (m.z[nb - 1] - m.z[0]);
            if (k > nz - nt) alphaz = m.pi * R4(0.005) * m.diml / m.dimc * (m.z[nz - 1] - m.z[k - 1]) / (m.z[nz - 1] - m.z[nz - nt]);
            double fdec00 = 1.0;
            for (long q = 0; q < NP; ++q) {
                long id = q + NP * (k - 1);
                double dampz = 0.0, fdec = 1.0;
                if (k < nb + 1) {
                    double r = (m.z[nb - 1] - m.z[k - 1]) / (m.z[nb - 1] - m.z[0]);
                    dampz = 3.0 * 3.0 * tempin[q] / (m.z[nb - 1] - m.z[0]) * (r * r);
                    fdec = alphaz / (dampz + alphaz);
                    m.gradp0_z[id] *= fdec; m.gradrho0_z[id] *= fdec;
                }
                if (k > nz - nt) {
                    double r = (m.z[nz - nt] - m.z[k - 1]) / (m.z[nz - 1] - m.z[nz - nt]);
                    dampz = 3.0 * 3.0 * tempin[q + NP * (long)(nz - 6)] / (m.z[nz - 1] - m.z[nz - nt]) * (r * r);
                    fdec = alphaz / (dampz + alphaz);
                    m.gradp0_z[id] *= fdec; m.gradrho0_z[id] *= fdec;
                }
                if (q == 0) fdec00 = fdec;
                m.bzpml[id] = -alphaz - dampz;
                m.az[id] = -dampz;
            }
            m.g[k - 1] = (k < nb + 1 || k > nz - nt) ? m.graw[k - 1] * fdec00 : m.graw[k - 1];
        }
    }
    m.gradrho0_x.assign(N, 0); m.gradp0_x.assign(N, 0); m.gradrho0_y.assign(N, 0); m.gradp0_y.assign(N, 0);
    ddx(m, m.rho0.data(), m.gradrho0_x.data());
    ddx(m, m.p0.data(), m.gradp0_x.data());
    // source planes: erad_2d = e_rad, orad_2d = o_rad (physics2d.f90:334-335)
    m.erad_2d.assign(NP, m.e_rad); m.orad_2d.assign(NP, m.o_rad); m.delta_width_2d.assign(NP, 0.0);
    for (long q = 0; q < NP; ++q) {
        const int k2 = m.P.compute_adjoint ? m.orad_2d[q] : m.erad_2d[q];
        m.delta_width_2d[q] = 2.0 / (m.z[k2] - m.z[k2 - 2]);
    }
    m.spongexyz.assign(N, 0.0);
}

// ----------------------------------------------------------------------------
// MP_MHD_PML_2D_DISPL (physics2d.f90:724-943), option 18 (ny = 1): PML at
// both ends with psi_vz, psi_p, psi_induction_bx, psi_dzbx; only the bottom
// row is zeroed
// ----------------------------------------------------------------------------
static void rhs_option18(Model& m) {
    long N = m.N, NP = m.NP; int nz = m.nz;
    double* xi_x = &m.temp_step[0]; double* xi_z = &m.temp_step[2 * N];
    double* v_x = &m.temp_step[3 * N]; double* v_z = &m.temp_step[5 * N];
    double* RHSxi_x = &m.scr[0]; double* RHSxi_z = &m.scr[2 * N];
    double* RHSv_x = &m.scr[3 * N]; double* RHSv_z = &m.scr[5 * N];
    long PS = NP * m.nzpml;
    double* psivz = &m.psipml[0]; double* psip = &m.psipml[PS];
    double* psidzbx = &m.psipml[2 * PS]; double* psiibx = &m.psipml[4 * PS];
    double* RHSpsivz = &m.scrpml[0]; double* RHSpsip = &m.scrpml[PS];
    double* RHSpsidzbx = &m.scrpml[2 * PS]; double* RHSpsiibx = &m.scrpml[4 * PS];
    int nb = m.P.npmlbot, nt = m.P.npmltop;
    std::vector<double> dxixdx(N), dxizdz(N, 0.0), p(N), rho(N), gradp_x(N), gradp_z(N, 0.0), flux2(N);
    std::vector<double> bx(N), bz(N), dzbx(N), curlby(N);
    auto pml = [&](double* deriv, double* psi, double* rhs) {
        int pmlindex = 0;
        for (int k = 1; k <= nz; ++k) {
            if (k <= nb || k >= nz - nt + 1) {
                pmlindex++;
                for (long q = 0; q < NP; ++q) {
                    long id = q + NP * (k - 1), ip = q + NP * (pmlindex - 1);
                    rhs[ip] = m.az[id] * deriv[id] + m.bzpml[id] * psi[ip];
                    deriv[id] = deriv[id] + psi[ip];
                }
            }
        }
    };
    ddx(m, xi_x, dxixdx.data());
    for (long q = 0; q < NP; ++q) dxizdz[q + NP * (nz - 1)] = -dxixdx[q + NP * (nz - 1)] * m.unstretch[nz - 1];
    oracle_dbyd2(dxizdz.data(), xi_z, NP, nz, 3);
    for (int k = 0; k < nz; ++k)
        for (long q = 0; q < NP; ++q) dxizdz[q + NP * k] *= m.stretch[k];
    pml(dxizdz.data(), psivz, RHSpsivz);
    for (long q = 0; q < N; ++q) {
        const double div = dxixdx[q] + dxizdz[q];
        p[q] = -m.c2rho0[q] * div - xi_z[q] * m.gradp0_z[q] - xi_x[q] * m.gradp0_x[q];
        rho[q] = -m.rho0[q] * div - xi_z[q] * m.gradrho0_z[q] - xi_x[q] * m.gradrho0_x[q];
    }
    ddx(m, p.data(), gradp_x.data());
    // ddz(p, gradp_z, 2): the caller-set bottom value is the previous
    // gradp_z(:,:,1), zero in every reachable state
    oracle_dbyd2(gradp_z.data(), p.data(), NP, nz, 2);
    for (int k = 0; k < nz; ++k)
        for (long q = 0; q < NP; ++q) gradp_z[q + NP * k] *= m.stretch[k];
    pml(gradp_z.data(), psip, RHSpsip);
    for (long q = 0; q < N; ++q) flux2[q] = -(xi_x[q] * m.boz[q] - xi_z[q] * m.box[q]);
    ddz(m, flux2.data(), bx.data(), 0);
    ddx(m, flux2.data(), bz.data());
    pml(bx.data(), psiibx, RHSpsiibx);
    for (long q = 0; q < N; ++q) bx[q] = -bx[q];
    ddz(m, bx.data(), dzbx.data(), 0);
    ddx(m, bz.data(), curlby.data());
    pml(dzbx.data(), psidzbx, RHSpsidzbx);
    for (long q = 0; q < N; ++q) {
        curlby[q] = -curlby[q] + dzbx[q];
        double flux1 = curlby[q] * m.boz[q];
        double flux3 = -curlby[q] * m.box[q];
        RHSv_x[q] = m.rhoinv[q] * (-gradp_x[q] + flux1);
        RHSv_z[q] = m.rhoinv[q] * (-gradp_z[q] + flux3);
        flux1 = m.curlboy[q] * bz[q];
        flux3 = -m.curlboy[q] * bx[q];
        RHSv_x[q] = RHSv_x[q] + m.rhoinv[q] * flux1;
        RHSv_z[q] = RHSv_z[q] + m.rhoinv[q] * flux3;
    }
    for (int k = 0; k < nz; ++k)
        for (long q = 0; q < NP; ++q) {
            long id = q + NP * k;
            RHSv_z[id] = RHSv_z[id] - m.rhoinv[id] * rho[id] * m.g[k];
        }
    for (long q = 0; q < N; ++q) { RHSxi_x[q] = v_x[q]; RHSxi_z[q] = v_z[q]; }
    if (m.P.damp_waves) {
        damp_velocity(m, v_x, RHSv_x);
        damp_velocity(m, v_z, RHSv_z);
    }
    if (m.src_mode != 0 && m.time <= m.forcing_length * m.cadforcing_step) {
        for (long q = 0; q < NP; ++q) {
            const int k2 = m.P.src_k > 0 ? m.P.src_k : (m.P.compute_adjoint ? m.orad_2d[q] : m.erad_2d[q]);
            long id = q + NP * (k2 - 1);
            if (m.P.compute_adjoint)
                RHSv_z[id] = RHSv_z[id] + m.forcing[q] * m.delta_width_2d[q] / m.rho0[id];
            else
                RHSv_z[id] = RHSv_z[id] + m.forcing[q] / m.rho0[id] * m.delta_width_2d[q];
        }
    }
    for (int l = 0; l < 6; ++l)
        for (long q = 0; q < NP; ++q) m.scr[l * N + q] = 0.0;
}

// ----------------------------------------------------------------------------
// MP_QUIET_PML_2D_DISPL (physics2d.f90:948-1105), option 17 (ny = 1)
// ----------------------------------------------------------------------------
static void rhs_option17(Model& m) {
    long N = m.N, NP = m.NP; int nz = m.nz;
    double* xi_x = &m.temp_step[0];
    double* xi_z = &m.temp_step[2 * N];
    double* v_x = &m.temp_step[3 * N];
    double* v_z = &m.temp_step[5 * N];
    double* RHSxi_x = &m.scr[0]; double* RHSxi_z = &m.scr[2 * N];
    double* RHSv_x = &m.scr[3 * N]; double* RHSv_z = &m.scr[5 * N];
    double* dxixdx = m.dvxdx.data(); double* dxizdz = m.gradvz.data();
    double* p = &m.scratch[N]; double* rho = &m.scratch[0];
    double* gradp_x = &m.gradp[0]; double* gradp_z = &m.gradp[2 * N];
    long PS = NP * m.nzpml;
    double* psivz = &m.psipml[0]; double* psip = &m.psipml[PS];
    double* RHSpsivz = &m.scrpml[0]; double* RHSpsip = &m.scrpml[PS];
    int nb = m.P.npmlbot, nt = m.P.npmltop;

    ddx(m, xi_x, dxixdx);
    for (long q = 0; q < NP; ++q)   // physics2d.f90:960 (caller-set top value, ibc=3)
        dxizdz[q + NP * (nz - 1)] = -dxixdx[q + NP * (nz - 1)] * m.unstretch[nz - 1];
    ddz(m, xi_z, dxizdz, 3);
    int pmlindex = 0;
    for (int k = 1; k <= nz; ++k)
        if (k <= nb || k >= nz - nt + 1) {
            pmlindex++;
            for (long q = 0; q < NP; ++q) {
                long id = q + NP * (k - 1), ip = q + NP * (pmlindex - 1);
                RHSpsivz[ip] = m.az[id] * dxizdz[id] + m.bzpml[id] * psivz[ip];
                dxizdz[id] = dxizdz[id] + psivz[ip];
            }
        }
    for (long q = 0; q < N; ++q) {
        m.div[q] = dxixdx[q] + dxizdz[q];
        p[q] = -m.c2rho0[q] * m.div[q] - m.gradp0_z[q] * xi_z[q];
    }
    ddx(m, p, gradp_x);
    // ibc=2: gradp_z(:,:,1) keeps its previous value (dbyd2.f90:130) -- it is the
    // value left by the previous call, which stays exactly zero for zero initial
    // state (the PML update at k=1 never makes it non-zero).
    ddz(m, p, gradp_z, 2);
    pmlindex = 0;
    for (int k = 1; k <= nz; ++k)
        if (k <= nb || k >= nz - nt + 1) {
            pmlindex++;
            for (long q = 0; q < NP; ++q) {
                long id = q + NP * (k - 1), ip = q + NP * (pmlindex - 1);
                RHSpsip[ip] = m.az[id] * gradp_z[id] + m.bzpml[id] * psip[ip];
                gradp_z[id] = gradp_z[id] + psip[ip];
            }
        }
    for (long q = 0; q < N; ++q) RHSv_x[q] = -m.rhoinv[q] * gradp_x[q];
    for (long q = 0; q < N; ++q) rho[q] = -m.rho0[q] * m.div[q] - m.gradrho0_z[q] * xi_z[q];
    for (int k = 0; k < nz; ++k)
        for (long q = 0; q < NP; ++q) {
            long id = q + NP * k;
            RHSv_z[id] = -m.rhoinv[id] * (gradp_z[id] + rho[id] * m.g[k]);
        }
    for (long q = 0; q < N; ++q) { RHSxi_x[q] = v_x[q]; RHSxi_z[q] = v_z[q]; }
    if (m.time <= m.forcing_length * m.cadforcing_step && m.src_mode != 0) {
        int ks = m.P.src_k > 0 ? m.P.src_k : (m.P.compute_adjoint ? m.o_rad : m.e_rad);
        for (long q = 0; q < NP; ++q) {
            long id = q + NP * (ks - 1);
            if (m.src_mode == 2)
                RHSv_z[id] = RHSv_z[id] + m.forcing[q] * m.delta_width / m.rho0[id];
            else
                RHSv_z[id] = RHSv_z[id] + m.forcing[q] * m.delta_width / m.rho0[id];
        }
    }
    for (long q = 0; q < NP; ++q) {
        RHSv_x[q] = 0.0; RHSv_z[q] = 0.0; RHSxi_x[q] = 0.0; RHSxi_z[q] = 0.0;
    }
}

// FILTER_VARS_3D (physics.f90:741-833)
static void filter_vars_3d(Model& m) {
    const double co[6] = {0.75390625, 0.41015625, -0.234375, 0.087890625, -0.01953125, 0.001953125};
    long NP = m.NP, N = m.N; int nz = m.nz;
#pragma omp parallel
    {
        std::vector<double> temp((long)nz);
#pragma omp for schedule(static)
        for (long lq = 0; lq < (long)m.dimfive * NP; ++lq) {
            int l = (int)(lq / NP); long q = lq % NP;
            double* A = &m.a[(long)l * N + q];
            auto av = [&](int k) { return A[NP * (long)(k - 1)]; };
            temp[1] = 0.5 * (av(3) + av(1));
            temp[2] = 0.5 * (av(4) + av(2));
            temp[3] = 0.5 * (av(5) + av(3));
            temp[4] = 0.5 * (av(6) + av(4));
            for (int k = 6; k <= nz - 5; ++k)
                temp[k - 1] = co[0] * av(k) + 0.5 * co[1] * (av(k - 1) + av(k + 1))
                            + 0.5 * co[2] * (av(k - 2) + av(k + 2))
                            + 0.5 * co[3] * (av(k - 3) + av(k + 3))
                            + 0.5 * co[4] * (av(k - 4) + av(k + 4))
                            + 0.5 * co[5] * (av(k - 5) + av(k + 5));
            temp[nz - 5] = 0.5 * (av(nz - 3) + av(nz - 5));
            temp[nz - 4] = 0.5 * (av(nz - 2) + av(nz - 4));
            temp[nz - 3] = 0.5 * (av(nz - 1) + av(nz - 3));
            temp[nz - 2] = 0.5 * (av(nz) + av(nz - 2));
            for (int k = 2; k <= nz - 1; ++k) A[NP * (long)(k - 1)] = temp[k - 1];
        }
    }
    if (m.time % m.freq_filtering == 0) {
        int nx = m.nx, ny = m.ny;
        for (int l = 0; l < 5; ++l) {
            double* A = &m.a[(long)l * N];
#pragma omp parallel
            {
                std::vector<cplx> spec(nx / 2 + 1), work;
#pragma omp for schedule(static)
                for (long row = 0; row < (long)ny * nz; ++row) {
                    r2c(A + row * nx, 1, nx, spec.data(), work);
                    for (int i = 0; i < nx / 2 + 1; ++i) spec[i] = spec[i] * m.decay_coeff_x[i];
                    c2r(spec.data(), nx, A + row * nx, 1, work);
                }
            }
#pragma omp parallel
            {
                std::vector<cplx> spec(ny / 2 + 1), work;
                std::vector<double> col(ny);
#pragma omp for schedule(static)
                for (long ik = 0; ik < (long)nx * nz; ++ik) {
                    long i = ik % nx, k = ik / nx;
                    for (int j = 0; j < ny; ++j) col[j] = A[IDX(m, i, j, k)];
                    r2c(col.data(), 1, ny, spec.data(), work);
                    for (int jj = 0; jj < ny / 2 + 1; ++jj) spec[jj] = spec[jj] * m.decay_coeff_y[jj];
                    c2r(spec.data(), ny, col.data(), 1, work);
                    for (int j = 0; j < ny; ++j) A[IDX(m, i, j, k)] = col[j];
                }
            }
        }
    }
}

// FILTER_VARS_2D (physics2d.f90:514-588): rows 2..5 are computed but not
// written back (kst stays 6); the spectral x filter runs when mod(time+1,30)=0
// on all six fields.
static void filter_vars_2d(Model& m) {
    const double co[6] = {0.75390625, 0.41015625, -0.234375, 0.087890625, -0.01953125, 0.001953125};
    long NP = m.NP, N = m.N; int nz = m.nz;
    std::vector<double> temp((long)nz);
    for (int l = 0; l < m.dimfive; ++l)
        for (long q = 0; q < NP; ++q) {
            double* A = &m.a[(long)l * N + q];
            auto av = [&](int k) { return A[NP * (long)(k - 1)]; };
            for (int k = 6; k <= nz - 5; ++k)
                temp[k - 1] = co[0] * av(k) + 0.5 * co[1] * (av(k - 1) + av(k + 1))
                            + 0.5 * co[2] * (av(k - 2) + av(k + 2))
                            + 0.5 * co[3] * (av(k - 3) + av(k + 3))
                            + 0.5 * co[4] * (av(k - 4) + av(k + 4))
                            + 0.5 * co[5] * (av(k - 5) + av(k + 5));
            temp[nz - 5] = 0.5 * (av(nz - 3) + av(nz - 5));
            temp[nz - 4] = 0.5 * (av(nz - 2) + av(nz - 4));
            temp[nz - 3] = 0.5 * (av(nz - 1) + av(nz - 3));
            temp[nz - 2] = 0.5 * (av(nz) + av(nz - 2));
            for (int k = 6; k <= nz - 1; ++k) A[NP * (long)(k - 1)] = temp[k - 1];
        }
    if ((m.time + 1) % m.freq_filtering == 0) {
        int nx = m.nx;
        std::vector<cplx> spec(nx / 2 + 1), work;
        for (int l = 0; l < m.dimfive; ++l) {
            double* A = &m.a[(long)l * N];
            for (long row = 0; row < (long)m.ny * nz; ++row) {
                r2c(A + row * nx, 1, nx, spec.data(), work);
                for (int i = 0; i < nx / 2 + 1; ++i) spec[i] = spec[i] * m.decay_coeff_x[i];
                c2r(spec.data(), nx, A + row * nx, 1, work);
            }
        }
    }
}

// LAGRANGE_INTERP (physics.f90:678-737), restated for the current time
static void lagrange_interp(Model& m) {
    double ts = R4(m.P.timestep), cad = R4(m.P.cadforcing);
    double xt = (double)m.time * ts / cad;
    int time1 = (int)std::floor(xt) + 1;
    xt = m.time * ts;
    double X[7];
    for (int l = 0; l < 7; ++l) X[l] = (double)(time1 - 4 + l) * cad;
    bool cond[7] = {X[0] >= 0, X[1] >= 0, X[2] >= 0, X[3] >= 0, true,
                    time1 < m.num_steps, time1 < m.num_steps - 1};
    long NP = m.NP;
    auto vrp = [&](int idx1) -> const double* {   // vr(:,:,idx1), 1-based, zero outside 1..L
        static thread_local std::vector<double> zero;
        if (idx1 >= 1 && idx1 <= m.vr_len) return &m.vr[(long)(idx1 - 1) * NP];
        zero.assign(NP, 0.0);
        return zero.data();
    };
    std::vector<double> den(7);
    for (int l = 0; l < 7; ++l) {
        double d = 1.0;
        for (int q = 0; q < 7; ++q) if (q != l) d = d * (X[l] - X[q]);
        den[l] = d;
    }
    for (long q = 0; q < NP; ++q) {
        double f = 0.0;
        for (int l = 0; l < 7; ++l) {
            double LC = cond[l] ? vrp(time1 - 3 + l)[q] / den[l] : 0.0;
            double t = LC;
            for (int r = 0; r < 7; ++r) if (r != l) t = t * (xt - X[r]);
            f = (l == 0) ? t : f + t;
        }
        m.forcing[q] = f;
    }
}

// STEP (step.f90:43-128) for options 2, 4 and 17 (USE_PML, no horizontal PML);
// in the velocity form the sixth field is unused and stays zero
static void step(Model& m) {
    long N6 = m.N * m.nf, NPML = (long)m.NP * m.nzpml * m.npv;
    for (int rk = 1; rk <= 5; ++rk) {
        if (rk == 1) {
            m.temp_step = m.a;
            for (long q = 0; q < NPML; ++q) m.psipml[q] = m.pmlvars[q];
        } else {
            double b = m.betas[rk - 1];
#pragma omp parallel for schedule(static)
            for (long q = 0; q < N6; ++q) m.temp_step[q] = m.a[q] + b * m.scr[q];
            for (long q = 0; q < NPML; ++q) m.psipml[q] = m.pmlvars[q] + b * m.scrpml[q];
        }
        if (m.P.option == 4) rhs_option4(m);
        else if (m.P.option == 2) rhs_option2(m);
        else if (m.P.option == 8) rhs_option8(m);
        else if (m.P.option == 10) rhs_option10(m);
        else if (m.P.option == 18) rhs_option18(m);
        else rhs_option17(m);
    }
#pragma omp parallel for schedule(static)
    for (long q = 0; q < N6; ++q) m.a[q] = m.a[q] + m.deltat * m.scr[q];
    for (long q = 0; q < NPML; ++q) m.pmlvars[q] = m.pmlvars[q] + m.deltat * m.scrpml[q];
    if (m.P.option == 17 || m.P.option == 18) filter_vars_2d(m);
    else filter_vars_3d(m);
}

// ----------------------------------------------------------------------------
// C API
// ----------------------------------------------------------------------------
extern "C" {

void* oracle_create(const oracle_params* P, const double* table) {
    try {
        Model* m = new Model();
        setup(*m, P, table);
        return m;
    } catch (...) { return nullptr; }
}

void oracle_destroy(void* h) { delete (Model*)h; }

int oracle_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n; return 1;
#endif
}

// Derived quantities (for tests): fills out[]; returns count written.
int oracle_info(void* h, double* out) {
    Model& m = *(Model*)h;
    int n = 0;
    out[n++] = m.e_rad; out[n++] = m.o_rad; out[n++] = m.delta_width; out[n++] = m.deltat;
    out[n++] = m.steps; out[n++] = m.freq_filtering; out[n++] = m.maxtime; out[n++] = m.forcing_length;
    out[n++] = m.cadforcing_step; out[n++] = m.num_steps;
    for (int i = 0; i < 5; ++i) out[n++] = m.betas[i];
    out[n++] = m.stretchx; out[n++] = m.stretchy; out[n++] = m.pi; out[n++] = m.rsun;
    out[n++] = m.dimc; out[n++] = m.dimrho; out[n++] = m.diml;
    return n;
}

// z-profiles used by the path (after PML modification): stretch, unstretch, g,
// gradp0_z, gradrho0_z, az, bzpml, rho0, c2 at (1,1,k)
int oracle_profiles(void* h, double* out /* 9*nz */) {
    Model& m = *(Model*)h;
    int nz = m.nz; long NP = m.NP;
    for (int k = 0; k < nz; ++k) {
        out[0 * nz + k] = m.stretch[k];
        out[1 * nz + k] = m.unstretch[k];
        out[2 * nz + k] = m.g[k];
        out[3 * nz + k] = m.gradp0_z[NP * k];
        out[4 * nz + k] = m.gradrho0_z[NP * k];
        out[5 * nz + k] = m.az[NP * k];
        out[6 * nz + k] = m.bzpml[NP * k];
        out[7 * nz + k] = m.rho0[NP * k];
        out[8 * nz + k] = m.c2[NP * k];
    }
    return 9 * nz;
}

int oracle_damping_rates(void* h, double* out) {
    Model& m = *(Model*)h;
    std::copy(m.damping_rates.begin(), m.damping_rates.end(), out);
    return (int)m.damping_rates.size();
}

// Source: planes (nx,ny,L) Fortran order; mode 1 = forward series, 2 = Lagrange.
int oracle_set_source(void* h, int mode, const double* planes, int L, const double* series, int nseries) {
    Model& m = *(Model*)h;
    m.src_mode = mode;
    m.vr.assign(planes, planes + (long)L * m.NP);
    m.vr_len = L;
    m.series.assign(series ? series : planes, series ? series + nseries : planes);
    return 0;
}

int oracle_set_state(void* h, const double* a, const double* pml) {
    Model& m = *(Model*)h;
    std::copy(a, a + m.N * m.nf, m.a.begin());
    if (pml) std::copy(pml, pml + (long)m.NP * m.nzpml * m.npv, m.pmlvars.begin());
    return 0;
}

int oracle_get_state(void* h, double* a, double* pml, double* scr) {
    Model& m = *(Model*)h;
    if (a) std::copy(m.a.begin(), m.a.end(), a);
    if (pml) std::copy(m.pmlvars.begin(), m.pmlvars.begin() + (long)m.NP * m.nzpml * m.npv, pml);
    if (scr) std::copy(m.scr.begin(), m.scr.end(), scr);
    return 0;
}

// One TIMESTEPPING iteration body (driver.f90:412-424) at time = m.time, then
// time advances.  Returns the current time index after the step.
int oracle_step(void* h, int nsteps) {
    Model& m = *(Model*)h;
    for (int s = 0; s < nsteps; ++s) {
        if (m.src_mode == 2) lagrange_interp(m);
        else if (m.src_mode == 1) {
            // forward series: forcing = plane0 * series(time); the 2-D reference
            // form uses vr(:,:,1) * fwdsource(time+1) (physics2d.f90:1066)
            double w = (m.time < (int)m.series.size()) ? m.series[m.time] : 0.0;
            for (long q = 0; q < m.NP; ++q) m.forcing[q] = m.vr[q] * w;
        }
        step(m);
        m.time++;
    }
    return m.time;
}

int oracle_set_time(void* h, int t) { ((Model*)h)->time = t; return 0; }

// MHD background of option 10 (3-D cgs arrays, (nz, ny, nx) C order)
int oracle_set_mhd(void* h, const double* rho, const double* c, const double* p, const double* bx,
                   const double* by, const double* bz) {
    Model& m = *(Model*)h;
    if (m.P.option != 10 && m.P.option != 8) return -1;
    setup_mhd(m, rho, c, p, bx, by, bz);
    return 0;
}

// 2-D MHD background of option 18 ((nz, nx) cgs: pressure, density, sound speed, vector potential)
static void setup_kernel_b2d(Model& m, const double* psi);

int oracle_set_mhd2d(void* h, const double* p, const double* rho, const double* c, const double* psi) {
    Model& m = *(Model*)h;
    if (m.P.option != 18) return -1;
    setup_mhd2d(m, p, rho, c, psi);
    setup_kernel_b2d(m, psi);
    return 0;
}

// MHD diagnostics: out = [box, boy, boz, curlbox, curlboy, curlboz, gradrho0_x, gradrho0_y,
// gradp0_x, gradp0_y, gradrho0_z, gradp0_z, az, bzpml, spongexyz] (15 * N)
int oracle_mhd_profiles(void* h, double* out) {
    Model& m = *(Model*)h;
    if (m.box.empty()) return -1;
    const std::vector<double>* v[15] = {&m.box, &m.boy, &m.boz, &m.curlbox, &m.curlboy, &m.curlboz,
                                        &m.gradrho0_x, &m.gradrho0_y, &m.gradp0_x, &m.gradp0_y,
                                        &m.gradrho0_z, &m.gradp0_z, &m.az, &m.bzpml, &m.spongexyz};
    for (int i = 0; i < 15; ++i) std::copy(v[i]->begin(), v[i]->end(), out + (long)i * m.N);
    return 0;
}

// Individual primitives, exposed for KATs and GPU parity tests.
int oracle_ddx(void* h, const double* var, double* dvar) { ddx(*(Model*)h, var, dvar); return 0; }
int oracle_ddy(void* h, const double* var, double* dvar) { ddy(*(Model*)h, var, dvar); return 0; }
int oracle_ddz(void* h, const double* var, double* dvar, int bc) { ddz(*(Model*)h, var, dvar, bc); return 0; }
int oracle_damp(void* h, const double* v, double* rhs) { damp_velocity(*(Model*)h, v, rhs); return 0; }

// FORWARD_SOURCE (driver.f90:1046-1071): Gabor wavelet sampled every timestep
int oracle_forward_source(const oracle_params* P, int nt, double* out) {
    double pi = R4(3.14159265358979), ts = R4(P->timestep);
    double nup = R4(P->nupeak), nuw = R4(P->nuwidth);
    for (int k = 1; k <= nt; ++k) {
        double tt = (double)((float)k - 1.0f) * ts;
        double arg = tt - 0.5 / nup;
        double f = std::cos(2.0 * pi * nup * tt) * std::exp(-2.0 * (arg * arg) * (nuw * nuw));
        if (std::fabs(f) < (double)0.00001f) f = 0.0;
        out[k - 1] = f * (double)1.0e-5f;
    }
    return nt;
}

// ----------------------------------------------------------------------------
// Sensitivity kernels (kernels.f90:197-311, scaling :523-539)
// ----------------------------------------------------------------------------
// FILTER_VAR_Z (kernels.f90:845-881)
static void filter_var_z(Model& m, double* var) {
    const double co[6] = {0.75390625, 0.41015625, -0.234375, 0.087890625, -0.01953125, 0.001953125};
    long NP = m.NP; int nz = m.nz;
#pragma omp parallel
    {
        std::vector<double> temp(nz);
#pragma omp for schedule(static)
        for (long q = 0; q < NP; ++q) {
            double* A = var + q;
            auto av = [&](int k) { return A[NP * (long)(k - 1)]; };
            temp[1] = 0.5 * (av(3) + av(1));
            temp[2] = 0.5 * (av(4) + av(2));
            temp[3] = 0.5 * (av(5) + av(3));
            temp[4] = 0.5 * (av(6) + av(4));
            for (int k = 6; k <= nz - 5; ++k)
                temp[k - 1] = co[0] * av(k) + 0.5 * co[1] * (av(k - 1) + av(k + 1))
                            + 0.5 * co[2] * (av(k - 2) + av(k + 2))
                            + 0.5 * co[3] * (av(k - 3) + av(k + 3))
                            + 0.5 * co[4] * (av(k - 4) + av(k + 4))
                            + 0.5 * co[5] * (av(k - 5) + av(k + 5));
            temp[nz - 5] = 0.5 * (av(nz - 3) + av(nz - 5));
            temp[nz - 4] = 0.5 * (av(nz - 2) + av(nz - 4));
            temp[nz - 3] = 0.5 * (av(nz - 1) + av(nz - 3));
            temp[nz - 2] = 0.5 * (av(nz) + av(nz - 2));
            for (int k = 2; k <= nz - 1; ++k) A[NP * (long)(k - 1)] = temp[k - 1];
        }
    }
}

// ddzkern (kernels.f90:609-621): dbyd2 * stretchkern, then FILTER_VAR_Z
static void ddzkern(Model& m, const double* var, double* dvar, int bc) {
    ddz(m, var, dvar, bc);
    filter_var_z(m, dvar);
}

// COMPUTE_DIV (kernels.f90:798-816)
static void compute_div(Model& m, const double* fx, const double* fy, const double* fz, double* dive) {
    std::vector<double> temp(m.N);
    ddx(m, fx, dive);
    if (m.ny > 4) {
        ddy(m, fy, temp.data());
        for (long q = 0; q < m.N; ++q) dive[q] = dive[q] + temp[q];
    }
    ddzkern(m, fz, temp.data(), 1);
    for (long q = 0; q < m.N; ++q) dive[q] = dive[q] + temp[q];
}

int oracle_kernel_reset(void* h) {
    Model& m = *(Model*)h;
    m.kernelc2.assign(m.N, 0.0); m.kernelrho.assign(m.N, 0.0); m.hessian.assign(m.N, 0.0);
    m.kernelb.assign(3 * m.N, 0.0);
    return 0;
}

// ---- magnetic kernels (kernels.f90:337-453, scaling :498-514) ---------------
// CROSS_KERN (kernels.f90:757-766): c = a x b on whole fields
static void cross_kern(const double* const a[3], const double* const b[3], double* const c[3], long N) {
    for (long q = 0; q < N; ++q) {
        const double cx = a[1][q] * b[2][q] - a[2][q] * b[1][q];
        const double cy = b[0][q] * a[2][q] - a[0][q] * b[2][q];
        const double cz = a[0][q] * b[1][q] - a[1][q] * b[0][q];
        c[0][q] = cx; c[1][q] = cy; c[2][q] = cz;
    }
}

// CURL_KERN (kernels.f90:770-793).  The boundary codes bcx, bcy, bcz are
// declared (initialize.f90:145) and never assigned; as module variables they
// are zero, so ddzkern takes bc 0.  ddykern of a 2-D box (ny = 1) multiplies
// by eyeky(1) = 0.
static void curl_kern(Model& m, const double* const f[3], double* const c[3]) {
    const long N = m.N;
    std::vector<double> temp(N);
    auto dy = [&](const double* v, double* d) {
        if (m.ny > 1) ddy(m, v, d);
        else std::fill(d, d + N, 0.0);
    };
    ddx(m, f[1], c[2]);
    dy(f[0], temp.data());
    for (long q = 0; q < N; ++q) c[2][q] = c[2][q] - temp[q];
    dy(f[2], c[0]);
    ddzkern(m, f[1], temp.data(), 0);
    for (long q = 0; q < N; ++q) c[0][q] = c[0][q] - temp[q];
    ddzkern(m, f[0], c[1], 0);
    ddx(m, f[2], temp.data());
    for (long q = 0; q < N; ++q) c[1][q] = c[1][q] - temp[q];
}

// B0 of kernel mode (kernels.f90:99-133): box = -ddzkern(psi, 0), boz =
// DBYD1(psi) stretchx (the solve's), both / dimb, boy = 0; curl B0 by CURL_KERN
static void setup_kernel_b2d(Model& m, const double* psi) {
    const long N = m.N;
    m.kbox.assign(N, 0.0);
    ddzkern(m, psi, m.kbox.data(), 0);
    for (long q = 0; q < N; ++q) m.kbox[q] = -m.kbox[q];
    for (long q = 0; q < N; ++q) m.kbox[q] = m.kbox[q] / m.dimb;
    m.kboz = m.boz;
    std::vector<double> zero(N, 0.0);
    m.kcurlbox.assign(N, 0.0); m.kcurlboy.assign(N, 0.0); m.kcurlboz.assign(N, 0.0);
    const double* f[3] = {m.kbox.data(), zero.data(), m.kboz.data()};
    double* c[3] = {m.kcurlbox.data(), m.kcurlboy.data(), m.kcurlboz.data()};
    curl_kern(m, f, c);
}

// One pass of the MAGNETIC_KERNELS block (kernels.f90:337-453): fxi = forward
// displacement (x, y, z), av = adjoint velocity (x, y, z), each N.
int oracle_kernel_accumulate_b(void* h, const double* fxi, const double* av) {
    Model& m = *(Model*)h;
    if (m.kbox.empty()) return -1;
    const long N = m.N;
    if (m.kernelb.size() != (size_t)(3 * N)) m.kernelb.assign(3 * N, 0.0);
    std::vector<double> buf(15 * N, 0.0);
    auto F = [&](int i) { return buf.data() + (long)i * N; };
    double* tx = F(0); double* ty = F(1); double* tz = F(2);
    double* fbx = F(3); double* fby = F(4); double* fbz = F(5);
    double* t1 = F(6); double* t2 = F(7); double* t3 = F(8);
    double* abx = F(9); double* aby = F(10); double* abz = F(11);
    std::vector<double> zero(N, 0.0);
    const double* xi[3] = {fxi, fxi + N, fxi + 2 * N};
    const double* va[3] = {av, av + N, av + 2 * N};
    const double* B0[3] = {m.kbox.data(), zero.data(), m.kboz.data()};
    const double* CB0[3] = {m.kcurlbox.data(), m.kcurlboy.data(), m.kcurlboz.data()};
    double* T[3] = {tx, ty, tz};
    double* T123[3] = {t1, t2, t3};
    double* FB[3] = {fbx, fby, fbz};
    double* AB[3] = {abx, aby, abz};
    const double* cT[3] = {tx, ty, tz};
    const double* cT123[3] = {t1, t2, t3};
    const double* cFB[3] = {fbx, fby, fbz};
    const double* cAB[3] = {abx, aby, abz};
    auto add = [&](const double* const v[3]) {
        for (int i = 0; i < 3; ++i)
            for (long q = 0; q < N; ++q) m.kernelb[(long)i * N + q] = m.kernelb[(long)i * N + q] + v[i][q];
    };
    cross_kern(xi, B0, T, N);
    curl_kern(m, cT, FB);
    curl_kern(m, cFB, T);
    cross_kern(va, cT, T123, N);
    add(cT123);
    // the first term
    cross_kern(cFB, va, T, N);
    curl_kern(m, cT, T123);
    add(cT123);
    // the third term
    cross_kern(va, B0, T, N);
    curl_kern(m, cT, AB);
    curl_kern(m, cAB, T);
    cross_kern(xi, cT, T123, N);
    add(cT123);
    // the second term
    cross_kern(va, CB0, T123, N);
    curl_kern(m, cT123, T);
    cross_kern(cT, xi, T123, N);
    add(cT123);
    // the fourth term: div(av) (COMPUTE_DIV), then (xi x curl B0) div(av)
    std::vector<double> dv(N);
    compute_div(m, va[0], va[1], va[2], dv.data());
    cross_kern(xi, CB0, T, N);
    for (int i = 0; i < 3; ++i)
        for (long q = 0; q < N; ++q) m.kernelb[(long)i * N + q] = m.kernelb[(long)i * N + q] + T[i][q] * dv[q];
    // equilibrium term 2: curl(B0 x (xi div(av)))
    for (int i = 0; i < 3; ++i)
        for (long q = 0; q < N; ++q) T[i][q] = xi[i][q] * dv[q];
    cross_kern(B0, cT, T123, N);
    curl_kern(m, cT123, T);
    add(cT);
    return 0;
}

// Scaling of the B-field kernels (kernels.f90:498-514): out = (kernel_bx,
// kernel_bz, kernel_vectorpsi), the last the y component of CURL_KERN of
// (kernel_bx, 0, kernel_bz).  2-D dimensions (test_in_2d).
int oracle_kernel_finish_b(void* h, double* out, int stepskern) {
    Model& m = *(Model*)h;
    if (m.kernelb.size() != (size_t)(3 * m.N)) return -1;
    const long N = m.N;
    const double ts = R4(m.P.timestep);
    const double dimen = 1.0 / (m.diml * (double)1.0e-8f * R4(m.P.xlength) * (double)1.0e-8f * m.dimb);
    std::vector<double> kb(3 * N);
    for (long q = 0; q < 3 * N; ++q) kb[q] = m.kernelb[q] * stepskern * ts * dimen;
    std::vector<double> zero(N, 0.0), cx(N), cy(N), cz(N);
    const double* f[3] = {kb.data(), zero.data(), kb.data() + 2 * N};
    double* c[3] = {cx.data(), cy.data(), cz.data()};
    curl_kern(m, f, c);
    std::copy(kb.begin(), kb.begin() + N, out);
    std::copy(kb.begin() + 2 * N, kb.end(), out + N);
    std::copy(cy.begin(), cy.end(), out + 2 * N);
    return 0;
}

// One accumulation of kernels.f90:276-311.  fwd = (xi_x, xi_y, xi_z, acc_x,
// acc_y, acc_z), adj = (v_x, v_y, v_z); each field is (nx,ny,nz).  The
// reference forces test_in_2d (kernels.f90:32), which zeroes every y term; a
// 3-D box (ny > 4) keeps them.  grav and c2 are the unmodified background.
int oracle_kernel_accumulate(void* h, const double* fwd, const double* adj, const double* grav_raw) {
    Model& m = *(Model*)h;
    long N = m.N, NP = m.NP; int nz = m.nz;
    const double *fxx = fwd, *fxy = fwd + N, *fxz = fwd + 2 * N;
    const double *fax = fwd + 3 * N, *fay = fwd + 4 * N, *faz = fwd + 5 * N;
    const double *avx = adj, *avy = adj + N, *avz = adj + 2 * N;
    std::vector<double> temp1(N), temp2(N), temp3(N), d31(N), d32(N, 0.0), d33(N);
    for (long q = 0; q < N; ++q)
        m.hessian[q] = m.hessian[q] + faz[q] * faz[q] + fax[q] * fax[q] + fay[q] * fay[q];
    compute_div(m, fxx, fxy, fxz, temp2.data());
    compute_div(m, avx, avy, avz, temp3.data());
    for (long q = 0; q < N; ++q) { temp1[q] = temp2[q] * temp3[q]; m.kernelc2[q] = m.kernelc2[q] + temp1[q]; }
    for (long q = 0; q < N; ++q)
        m.kernelrho[q] = m.kernelrho[q] + temp1[q] * m.c2[q] + faz[q] * avz[q] + fax[q] * avx[q] + fay[q] * avy[q];
    for (int k = 0; k < nz; ++k)
        for (long q = 0; q < NP; ++q) temp2[q + NP * k] = avz[q + NP * k] * grav_raw[k];
    ddx(m, temp2.data(), d31.data());
    if (m.ny > 4) ddy(m, temp2.data(), d32.data());
    ddzkern(m, temp2.data(), d33.data(), 1);
    for (int k = 0; k < nz; ++k)
        for (long q = 0; q < NP; ++q) {
            long id = q + NP * k;
            m.kernelrho[id] = m.kernelrho[id] - grav_raw[k] * fxz[id] * temp3[id]
                + (fxx[id] * d31[id] + fxy[id] * d32[id] + fxz[id] * d33[id]);
        }
    return 0;
}

// Final scaling (kernels.f90:523-539).  out = (kernel_c, kernel_rho, hessian).
int oracle_kernel_finish(void* h, double* out, int stepskern) {
    Model& m = *(Model*)h;
    long N = m.N;
    double ts = R4(m.P.timestep);
    double dimen = std::pow(m.diml * (double)1.0e-8f, -3.0);
    if (m.ny <= 4)
        dimen = 1.0 / (m.diml * (double)1.0e-8f * R4(m.P.xlength) * (double)1.0e-8f);
    for (long q = 0; q < N; ++q) {
        double r0 = m.rho0[q], c2 = m.c2[q];
        out[q] = -m.kernelc2[q] * r0 * c2 * stepskern * ts * dimen * 2.0;
        out[N + q] = -r0 * m.kernelrho[q] * stepskern * ts * dimen;
        out[2 * N + q] = m.hessian[q];
    }
    return 0;
}

// Spectral view helpers for tests: plane r2c of one (nx,ny) plane (unnormalised)
int oracle_plane_r2c(void* h, const double* in, double* out_interleaved) {
    Model& m = *(Model*)h;
    int hh = m.nx / 2 + 1;
    std::vector<cplx> spec((long)hh * m.ny);
    plane_r2c(m, in, spec.data());
    for (long q = 0; q < (long)hh * m.ny; ++q) { out_interleaved[2 * q] = spec[q].real(); out_interleaved[2 * q + 1] = spec[q].imag(); }
    return 0;
}

}  // extern "C"
