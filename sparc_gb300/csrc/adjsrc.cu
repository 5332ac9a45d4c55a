// Adjoint source of a 2-D run on the GPU: ADJOINT_SOURCE_FILT
// (driver.f90:1262-1686) with the ridge filters FMODE_FILTER / PMODE_FILTER
// (driver.f90:1074-1119, 1173-1222), FREQ_FILTER (:1225-1237) and
// COMPUTE_TT (:921-960).
//
// The surface records stay on the device between the forward and the adjoint
// solves.  Transforms along t (nt outputs, any length) and along x are direct
// FP64 DFTs with exact twiddle tables: at nx = 256 and nt = 481 one 2-D
// transform is 7e7 complex multiply-adds.  The reference back-propagates each
// measurement with its own inverse 2-D FFT and adds the real part to the
// adjoint source; the transform is linear, so here every receiver's windowed,
// weighted spectrum is summed in (k, nu) first and each filter set needs one
// inverse transform.
#include <cmath>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "adjsrc.cuh"

namespace {

inline double r4(double v) { return (double)(float)v; }
const double PI_R4 = r4(3.14159265358979);      // initialize.f90:38

// distmat (initialize.f90:1124-1141): signed index distance
double distmat_at(int i1, int n) {              // i1 = 1-based index
    const int i2 = std::min(i1 - 1, n - i1 + 1);
    return (i1 - 1 > n - i1 + 1) ? -(double)i2 : (double)i2;
}

void ridge_filter(std::vector<double>& out, int nx, int nt, double xlength, double outputcad, bool fm) {
    // FMODE_FILTER / PMODE_FILTER: raised cosine between f0 = c k^0.5 and the
    // polynomial ridge f1, tapered below f_low + df (f in mHz)
    const double c = fm ? r4(2.056565) : r4(3.96);
    const double p0 = fm ? 1.0 : r4(1.1), p1 = fm ? 3.0 : r4(5.2), p2 = fm ? r4(-0.6) : r4(-1.3);
    const double df = 0.5, f_low = fm ? r4(1.1) : r4(1.6);
    out.assign((size_t)nt * nx, 0.0);
    std::vector<double> k(nx), f(nt);
    for (int i = 0; i < nx; ++i)
        k[i] = std::fabs(distmat_at(i + 1, nx)) * 2.0 * PI_R4 / (xlength * r4(1e-8) * nx / (nx - 1.0));
    for (int j = 0; j < nt; ++j) {
        const double w = std::fabs(distmat_at(j + 1, nt)) * 2.0 * PI_R4 / (nt * outputcad);
        f[j] = w / (2.0 * PI_R4) * 1e3;
    }
    for (int i = 0; i < nx; ++i) {
        const double f0 = c * std::pow(fm ? k[i] : std::fabs(k[i]), 0.5);
        const double f1 = p0 + p1 * k[i] + p2 * std::pow(k[i], 2.0);
        const double delta = f1 - f0;
        for (int j = 0; j < nt; ++j) {
            const double d = f[j] - f0;
            if (d < delta && d > 0) out[(size_t)j * nx + i] = 0.5 * (1.0 + std::cos(PI_R4 * (2.0 * d / delta - 1)));
        }
    }
    for (int j = 0; j < nt; ++j) {
        const double taper = 0.5 * (1.0 + std::cos(PI_R4 * (f[j] - (f_low + df)) / df));
        for (int i = 0; i < nx; ++i) {
            double& v = out[(size_t)j * nx + i];
            if (fm) {
                if (f[j] < f_low + df) v = v * taper;
                if (f[j] < f_low) v = 0.0;
            } else {
                if (f[j] < f_low) v = 0.0;
                if (f[j] < f_low + df) v = v * taper;
            }
        }
    }
}

std::vector<double> freq_filter(double f1, double f2, int nt, double outputcad) {
    std::vector<double> w(nt), filt(nt);
    for (int j = 0; j < nt; ++j) w[j] = std::fabs(distmat_at(j + 1, nt)) * 1e3 / (nt * outputcad);
    const double wid = r4(0.4) * (w[1] - w[0]);
    for (int j = 0; j < nt; ++j) filt[j] = 1.0 / (1.0 + std::exp((f1 - w[j]) / wid)) - 1.0 / (1.0 + std::exp((f2 - w[j]) / wid));
    return filt;
}

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// direct DFT along one axis: out[o][q] = sum_p in[o][p] W^(sign p q) with the
// axis of length n at element stride st and the other of length m at stride
// so; in may be real (real_in) or complex
__global__ void dft_axis_kernel(const double2* __restrict__ in, const double* __restrict__ in_re, double2* __restrict__ out,
                                int n, int m, long long st, long long so, const double2* __restrict__ W, int sign) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)n * m) return;
    // the other axis fastest across threads when the transform axis is the
    // slow one (coalesced reads of a row)
    const int o = (int)(so == 1 ? t % m : t / n), q = (int)(so == 1 ? t / m : t % n);
    double2 acc = make_double2(0.0, 0.0);
    for (int p = 0; p < n; ++p) {
        const long long idx = (long long)p * st + (long long)o * so;
        const double2 v = in_re ? make_double2(in_re[idx], 0.0) : in[idx];
        double2 w = W[(int)(((long long)p * q) % n)];
        if (sign > 0) w.y = -w.y;
        acc = make_double2(acc.x + (v.x * w.x - v.y * w.y), acc.y + (v.x * w.y + v.y * w.x));
    }
    out[(long long)q * st + (long long)o * so] = acc;
}

__global__ void spec_filter_kernel(double2* __restrict__ out, const double2* __restrict__ in, const double* __restrict__ filt,
                                   const double* __restrict__ dmul, int nx, long long n) {
    // out = in * filt (and * (i nu 2 pi) when dmul, the time derivative)
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    double2 v = in[t];
    v.x *= filt[t]; v.y *= filt[t];
    if (dmul) {
        const double d = dmul[t / nx];
        v = make_double2(-v.y * d, v.x * d);
    }
    out[t] = v;
}

struct RecvArgs {
    int nx, nt, mode, linesearch;
    double dt, t1, x0, xlength;
    double mindist, maxdist;
    int halftime;
    double vel[2];         // ridge speeds of sets 0, 1 (Mm/min)
    double pc[5];          // arrival polynomial of set 2 (min, Mm)
    int spectrum;          // 1: the windowed spectrum for the adjoint source; 0: tau only
};

// one CTA per pixel i: window, COMPUTE_TT, ||ccdot||^2 and the windowed
// spectrum of the time derivative times -tau / (||ccdot||^2 dt)
__global__ void receiver_kernel(RecvArgs a, const double2* __restrict__ A, const double2* __restrict__ D,
                                const double2* __restrict__ C, const double2* __restrict__ Wt, int* __restrict__ win,
                                double2* __restrict__ R, double* __restrict__ tau_out, int* __restrict__ flag,
                                int* __restrict__ err) {
    extern __shared__ double cc[];                 // 2 nt - 1 lags
    __shared__ int s_lef, s_rig, s_active;
    __shared__ double s_tau;
    __shared__ double2 s_con;
    const int i = blockIdx.x, nx = a.nx, nt = a.nt;
    if (threadIdx.x == 0) {
        const double x = (double)i / nx;
        const double d = fabs((x - 0.5) * a.xlength * (double)1.0e-8f - a.x0);
        s_active = (d > a.mindist && d < a.maxdist) ? 1 : 0;
        int lef = 0, rig = 0;
        if (s_active) {
            int loc = 0;
            if (a.mode < 2 && a.linesearch) {
                lef = win[2 * i];
                rig = win[2 * i + 1];
            } else if (a.mode < 2) {
                const double vel = a.vel[a.mode];
                const int timest = (int)floor(d / vel * 1.0 / a.dt), timefin = timest + 40;
                if (timest < 1 || timefin > nt) { atomicExch(err, 1); s_active = 0; }
                else {
                    double best = -1.0;
                    for (int t = timest; t <= timefin; ++t) {
                        const double v = fabs(A[(long long)(t - 1) * nx + i].x);
                        if (v > best) { best = v; loc = t; }
                    }
                }
            } else if (d < 250.0) {
                const double v = (a.pc[0] - a.t1 + a.pc[1] * d + a.pc[2] * pow(d, 2.0) + a.pc[3] * pow(d, 3.0) +
                                  a.pc[4] * pow(d, 4.0)) / a.dt;
                const int tsm = (v >= 0 ? (int)floor(v + 0.5) : -(int)floor(-v + 0.5)) + 1;
                if (tsm - 6 < 1 || tsm + 6 > nt) { atomicExch(err, 1); s_active = 0; }
                else {
                    double best = -1e300;
                    for (int t = tsm - 6; t <= tsm + 6; ++t) {
                        const double v2 = A[(long long)(t - 1) * nx + i].x;
                        if (v2 > best) { best = v2; loc = t; }
                    }
                }
            } else {
                double best = -1e300;
                for (int t = 1; t <= nt; ++t) {
                    const double v2 = A[(long long)(t - 1) * nx + i].x;
                    if (v2 > best) { best = v2; loc = t; }
                }
            }
            if (s_active && !(a.mode < 2 && a.linesearch)) { lef = loc - a.halftime; rig = loc + a.halftime; }
            if (s_active && (lef < 1 || rig > nt || rig < lef)) { atomicExch(err, 2); s_active = 0; }
        }
        s_lef = lef;
        s_rig = rig;
        if (a.mode < 2 && !a.linesearch) { win[2 * i] = s_active ? lef : 0; win[2 * i + 1] = s_active ? rig : 0; }
    }
    __syncthreads();
    if (!s_active) {
        if (a.spectrum)                            // R (and C) exist only when the spectrum is formed
            for (int q = threadIdx.x; q < nt; q += blockDim.x) R[(long long)i * nt + q] = make_double2(0.0, 0.0);
        if (threadIdx.x == 0) { flag[i] = 0; tau_out[i] = 0.0; }
        return;
    }
    const int lef = s_lef, leng = s_rig - s_lef + 1;
    // COMPUTE_TT: cc over lags -leng+1..leng-1, each a sequential sum
    for (int l = threadIdx.x; l < 2 * leng - 1; l += blockDim.x) {
        const int lag = l - (leng - 1);
        double s = 0.0;
        if (lag <= 0) {
            const int l1 = -lag;                    // 0-based start in u0
            for (int q = 0; q < leng - l1; ++q)
                s = s + A[(long long)(lef - 1 + l1 + q) * nx + i].x * D[(long long)(lef - 1 + q) * nx + i].x;
        } else {
            for (int q = 0; q < leng - lag; ++q)
                s = s + A[(long long)(lef - 1 + q) * nx + i].x * D[(long long)(lef - 1 + lag + q) * nx + i].x;
        }
        cc[l] = s * a.dt;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int loc = 0;
        double best = cc[0];
        for (int l = 1; l < 2 * leng - 1; ++l)
            if (cc[l] > best) { best = cc[l]; loc = l; }
        double tau = 0.0;
        if (loc < 1 || loc > 2 * leng - 3) {
            atomicExch(err, 3);
        } else {
            // the quadratic through the peak: `inverse` (driver.f90:964-1042),
            // Doolittle LU of [1 t t^2] and one solve per column
            double m[3][3], L[3][3] = {{0}}, U[3][3] = {{0}}, inv[3][3];
            for (int r = 0; r < 3; ++r) {
                const double tt = (double)(loc - 1 + r - (leng - 1)) * a.dt;
                m[r][0] = 1.0; m[r][1] = tt; m[r][2] = pow(tt, 2.0);
            }
            for (int k = 0; k < 2; ++k)
                for (int r = k + 1; r < 3; ++r) {
                    const double coeff = m[r][k] / m[k][k];
                    L[r][k] = coeff;
                    for (int j = k + 1; j < 3; ++j) m[r][j] = m[r][j] - coeff * m[k][j];
                }
            for (int r = 0; r < 3; ++r) L[r][r] = 1.0;
            for (int j = 0; j < 3; ++j)
                for (int r = 0; r <= j; ++r) U[r][j] = m[r][j];
            for (int k = 0; k < 3; ++k) {
                double b[3] = {0, 0, 0}, dd[3], xx[3];
                b[k] = 1.0;
                dd[0] = b[0];
                for (int r = 1; r < 3; ++r) {
                    dd[r] = b[r];
                    for (int j = 0; j < r; ++j) dd[r] = dd[r] - L[r][j] * dd[j];
                }
                xx[2] = dd[2] / U[2][2];
                for (int r = 1; r >= 0; --r) {
                    xx[r] = dd[r];
                    for (int j = 2; j > r; --j) xx[r] = xx[r] - U[r][j] * xx[j];
                    xx[r] = xx[r] / U[r][r];
                }
                for (int r = 0; r < 3; ++r) inv[r][k] = xx[r];
            }
            const double p1 = inv[1][0] * cc[loc - 1] + inv[1][1] * cc[loc] + inv[1][2] * cc[loc + 1];
            const double p2 = inv[2][0] * cc[loc - 1] + inv[2][1] * cc[loc] + inv[2][2] * cc[loc + 1];
            tau = -p1 * 0.5 / p2;
        }
        s_tau = tau;
        tau_out[i] = tau;
        flag[i] = 1;
    }
    __syncthreads();
    if (!a.spectrum) return;
    if (threadIdx.x == 0) {
        // sum(ccdot(i,1,lef:rig)**2.) of the complex derivative
        double2 nrm = make_double2(0.0, 0.0);
        for (int t = lef; t <= s_rig; ++t) {
            const double2 cv = C[(long long)(t - 1) * nx + i];
            nrm = make_double2(nrm.x + (cv.x * cv.x - cv.y * cv.y), nrm.y + 2.0 * cv.x * cv.y);
        }
        const double2 den = make_double2(nrm.x * a.dt, nrm.y * a.dt);
        const double q2 = den.x * den.x + den.y * den.y;
        const double tau = s_tau;
        s_con = make_double2(-tau * den.x / q2, tau * den.y / q2);      // -tau / den
    }
    __syncthreads();
    // the windowed time derivative's spectrum (1-D DFT over t), times con
    const double2 con = s_con;
    for (int q = threadIdx.x; q < nt; q += blockDim.x) {
        double2 acc = make_double2(0.0, 0.0);
        for (int t = lef; t <= s_rig; ++t) {
            const double2 v = C[(long long)(t - 1) * nx + i];
            const double2 w = Wt[(int)(((long long)(t - 1) * q) % nt)];
            acc = make_double2(acc.x + (v.x * w.x - v.y * w.y), acc.y + (v.x * w.y + v.y * w.x));
        }
        R[(long long)i * nt + q] = cmul(con, acc);
    }
}

// S(nu, k) = sum over measured pixels i of filt(nu, k) R_i(nu) exp(-i 2 pi kk x_i)
__global__ void back_project_kernel(double2* __restrict__ S, const double* __restrict__ filt, const double2* __restrict__ R,
                                    const int* __restrict__ flag, const double* __restrict__ kk, int nx, int nt) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)nx * nt) return;
    const int nu = (int)(t / nx), k = (int)(t % nx);
    const double f = filt[t];
    const double base = kk[k] * 2.0 * (double)3.14159265358979f;
    double2 acc = make_double2(0.0, 0.0);
    for (int i = 0; i < nx; ++i) {
        if (!flag[i]) continue;
        double sn, cs;
        sincos(base * ((double)i / nx), &sn, &cs);
        const double2 r = R[(long long)i * nt + nu];
        const double2 fr = make_double2(f * r.x, f * r.y);
        const double2 e = make_double2(cs, -sn);
        const double2 v = cmul(fr, e);
        acc = make_double2(acc.x + v.x, acc.y + v.y);
    }
    S[t] = acc;
}

// adj(nt-1-t, x) += Re(field(t, x))
__global__ void reverse_add_kernel(double* __restrict__ adj, const double2* __restrict__ f, int nx, int nt) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)nx * nt) return;
    const int tt = (int)(t / nx), x = (int)(t % nx);
    adj[(long long)(nt - 1 - tt) * nx + x] += f[t].x;
}

__global__ void scale_kernel(double* a, double s, long long n) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) a[t] = a[t] * s;
}

unsigned nbk(long long n) { return (unsigned)((n + 255) / 256); }

struct DevBuf {
    std::vector<void*> ptrs;
    cudaError_t err = cudaSuccess;
    template <typename T> T* get(size_t count) {
        void* p = nullptr;
        cudaError_t e = cudaMalloc(&p, count * sizeof(T));
        if (e != cudaSuccess) { err = e; cudaGetLastError(); return nullptr; }
        ptrs.push_back(p);
        return (T*)p;
    }
    ~DevBuf() { for (void* p : ptrs) cudaFree(p); }
};

}  // namespace

int adjsrc_compute(cudaStream_t s, const double* acc_dev, const double* dat_host, int nt, int nx, double xlength,
                   double outputcad, const AdjSrcArgs& a, int* windows, double* adj_host, double* misfit,
                   int* nmeas, std::string& why) {
    if (nt < 8 || nx < 4) { why = "need at least 8 outputs and 4 pixels"; return 1; }
    if (nt > 12000) { why = "more than 12000 outputs"; return 1; }
    const long long n = (long long)nt * nx;
    // host tables (FP64): filters, twiddles, signed wave numbers, frequencies
    std::vector<double> fmode, pmode;
    ridge_filter(fmode, nx, nt, xlength, outputcad, true);
    ridge_filter(pmode, nx, nt, xlength, outputcad, false);
    std::vector<double> filt(nt, 1.0);
    if (a.have_band[0]) filt = freq_filter(a.band[0][0], a.band[0][1], nt, outputcad);
    for (int j = 0; j < nt; ++j)
        for (int i = 0; i < nx; ++i) fmode[(size_t)j * nx + i] *= filt[j];
    if (a.have_band[1]) filt = freq_filter(a.band[1][0], a.band[1][1], nt, outputcad);
    for (int j = 0; j < nt; ++j)
        for (int i = 0; i < nx; ++i) pmode[(size_t)j * nx + i] *= filt[j];
    std::vector<double> highp((size_t)n);
    for (int j = 0; j < nt; ++j)
        for (int i = 0; i < nx; ++i) highp[(size_t)j * nx + i] = 1.0 * filt[j];
    std::vector<double> Wt(2 * nt), Wx(2 * nx), kk(nx), dmul(nt);
    for (int q = 0; q < nt; ++q) { Wt[2 * q] = std::cos(2.0 * M_PI * q / nt); Wt[2 * q + 1] = -std::sin(2.0 * M_PI * q / nt); }
    for (int q = 0; q < nx; ++q) { Wx[2 * q] = std::cos(2.0 * M_PI * q / nx); Wx[2 * q + 1] = -std::sin(2.0 * M_PI * q / nx); }
    for (int i = 0; i < nx; ++i) kk[i] = distmat_at(i + 1, nx);
    for (int j = 0; j < nt; ++j) dmul[j] = distmat_at(j + 1, nt) / (nt * a.dt * 60.0) * (2.0 * PI_R4);
    DevBuf B;
    double2 *d_Wt = B.get<double2>(nt), *d_Wx = B.get<double2>(nx);
    double *d_kk = B.get<double>(nx), *d_dmul = B.get<double>(nt), *d_dat = B.get<double>(n), *d_filt = B.get<double>(n);
    double2 *spec = B.get<double2>(n), *specd = B.get<double2>(n), *tmp = B.get<double2>(n), *tmp2 = B.get<double2>(n);
    double2 *A = B.get<double2>(n), *D = B.get<double2>(n), *C = B.get<double2>(n), *R = B.get<double2>(n);
    double *d_adj = B.get<double>(n), *d_tau = B.get<double>(nx);
    int *d_flag = B.get<int>(nx), *d_win = B.get<int>(2 * nx), *d_err = B.get<int>(1);
    if (B.err != cudaSuccess) { why = std::string("device allocation: ") + cudaGetErrorString(B.err); return 2; }
    cudaMemcpyAsync(d_Wt, Wt.data(), nt * 16, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(d_Wx, Wx.data(), nx * 16, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(d_kk, kk.data(), nx * 8, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(d_dmul, dmul.data(), nt * 8, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(d_dat, dat_host, n * 8, cudaMemcpyHostToDevice, s);
    cudaMemsetAsync(d_adj, 0, n * 8, s);
    cudaMemsetAsync(d_err, 0, 4, s);
    // 2-D transforms of (nt, nx) fields: along t (stride nx, threads over x),
    // then along x (stride 1)
    auto dft2 = [&](const double2* in, const double* in_re, double2* out, int sign) {
        dft_axis_kernel<<<nbk(n), 256, 0, s>>>(in, in_re, tmp2, nt, nx, nx, 1, d_Wt, sign);
        dft_axis_kernel<<<nbk(n), 256, 0, s>>>(tmp2, nullptr, out, nx, nt, 1, nx, d_Wx, sign);
    };
    dft2(nullptr, acc_dev, spec, -1);
    dft2(nullptr, d_dat, specd, -1);
    double sum_tau2 = 0.0;
    int count = 0;
    const double* filters[3] = {fmode.data(), pmode.data(), highp.data()};
    for (int mode = 0; mode < 3; ++mode) {
        if (!a.have_ridge[mode]) continue;
        cudaMemcpyAsync(d_filt, filters[mode], n * 8, cudaMemcpyHostToDevice, s);
        spec_filter_kernel<<<nbk(n), 256, 0, s>>>(tmp, spec, d_filt, nullptr, nx, n);
        dft2(tmp, nullptr, A, +1);
        spec_filter_kernel<<<nbk(n), 256, 0, s>>>(tmp, specd, d_filt, nullptr, nx, n);
        dft2(tmp, nullptr, D, +1);
        spec_filter_kernel<<<nbk(n), 256, 0, s>>>(tmp, spec, d_filt, d_dmul, nx, n);
        dft2(tmp, nullptr, C, +1);
        RecvArgs ra;
        ra.nx = nx; ra.nt = nt; ra.mode = mode; ra.linesearch = (mode < 2 && a.linesearch) ? 1 : 0;
        ra.dt = a.dt; ra.t1 = a.t1; ra.x0 = a.x00; ra.xlength = xlength;
        ra.mindist = a.ridge[mode][0]; ra.maxdist = a.ridge[mode][1];
        ra.halftime = (int)std::floor(a.ridge[mode][2] / (2.0 * a.dt) + 0.5);
        ra.vel[0] = 0.75; ra.vel[1] = 1.00;                        // driver.f90:1461-1462
        const double pc[5] = {r4(13.4090), r4(0.3421), r4(-0.0005), 0.0, 0.0};   // driver.f90:1557-1559
        for (int q = 0; q < 5; ++q) ra.pc[q] = pc[q];
        ra.spectrum = 1;
        if (mode < 2) cudaMemcpyAsync(d_win, windows + (size_t)mode * 2 * nx, 2 * nx * sizeof(int),
                                      cudaMemcpyHostToDevice, s);
        const size_t smc = (size_t)(2 * nt) * 8;
        if (smc > 48 * 1024) cudaFuncSetAttribute((const void*)receiver_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                  (int)smc);
        receiver_kernel<<<nx, 128, smc, s>>>(ra, A, D, C, d_Wt, d_win, R, d_tau, d_flag, d_err);
        back_project_kernel<<<nbk(n), 256, 0, s>>>(tmp, d_filt, R, d_flag, d_kk, nx, nt);
        dft2(tmp, nullptr, A, +1);
        reverse_add_kernel<<<nbk(n), 256, 0, s>>>(d_adj, A, nx, nt);
        std::vector<double> tau(nx);
        std::vector<int> flag(nx);
        cudaMemcpyAsync(tau.data(), d_tau, nx * 8, cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(flag.data(), d_flag, nx * 4, cudaMemcpyDeviceToHost, s);
        if (mode < 2 && !a.linesearch)
            cudaMemcpyAsync(windows + (size_t)mode * 2 * nx, d_win, 2 * nx * sizeof(int), cudaMemcpyDeviceToHost, s);
        if (cudaStreamSynchronize(s) != cudaSuccess) {
            why = std::string("CUDA error: ") + cudaGetErrorString(cudaGetLastError());
            return 2;
        }
        for (int i = 0; i < nx; ++i)
            if (flag[i]) { sum_tau2 = sum_tau2 + std::pow(tau[i], 2.0); ++count; }
    }
    scale_kernel<<<nbk(n), 256, 0, s>>>(d_adj, (double)nt / 60.0, n);
    int herr = 0;
    cudaMemcpyAsync(adj_host, d_adj, n * 8, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(&herr, d_err, 4, cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) {
        why = std::string("CUDA error: ") + cudaGetErrorString(cudaGetLastError());
        return 2;
    }
    if (herr) {
        why = herr == 1 ? "a measurement window starts or ends outside the record"
                        : (herr == 2 ? "a window [lef, rig] lies outside the record"
                                     : "a cross-correlation peak sits at the end of the lag range");
        return 1;
    }
    *misfit = 0.5 * sum_tau2;
    *nmeas = count;
    return 0;
}

int misfit_all_compute(cudaStream_t s, const double* acc_dev, const double* dat_host, int nt, int nx, double xlength,
                       double outputcad, const AdjSrcArgs& a, int* windows, double* misfit, int* nmeas,
                       std::string& why) {
    if (nt < 8 || nx < 4) { why = "need at least 8 outputs and 4 pixels"; return 1; }
    if (nt > 12000) { why = "more than 12000 outputs"; return 1; }
    const long long n = (long long)nt * nx;
    std::vector<double> fm0, pm0;
    ridge_filter(fm0, nx, nt, xlength, outputcad, true);
    ridge_filter(pm0, nx, nt, xlength, outputcad, false);
    std::vector<double> Wt(2 * nt), Wx(2 * nx);
    for (int q = 0; q < nt; ++q) { Wt[2 * q] = std::cos(2.0 * M_PI * q / nt); Wt[2 * q + 1] = -std::sin(2.0 * M_PI * q / nt); }
    for (int q = 0; q < nx; ++q) { Wx[2 * q] = std::cos(2.0 * M_PI * q / nx); Wx[2 * q + 1] = -std::sin(2.0 * M_PI * q / nx); }
    DevBuf B;
    double2 *d_Wt = B.get<double2>(nt), *d_Wx = B.get<double2>(nx);
    double *d_dat = B.get<double>(n), *d_filt = B.get<double>(n), *d_tau = B.get<double>(nx);
    double2 *spec = B.get<double2>(n), *specd = B.get<double2>(n), *tmp = B.get<double2>(n), *tmp2 = B.get<double2>(n);
    double2 *A = B.get<double2>(n), *D = B.get<double2>(n);
    int *d_flag = B.get<int>(nx), *d_win = B.get<int>(2 * nx), *d_err = B.get<int>(1);
    if (B.err != cudaSuccess) { why = std::string("device allocation: ") + cudaGetErrorString(B.err); return 2; }
    cudaMemcpyAsync(d_Wt, Wt.data(), nt * 16, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(d_Wx, Wx.data(), nx * 16, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(d_dat, dat_host, n * 8, cudaMemcpyHostToDevice, s);
    cudaMemsetAsync(d_err, 0, 4, s);
    auto dft2 = [&](const double2* in, const double* in_re, double2* out, int sign) {
        dft_axis_kernel<<<nbk(n), 256, 0, s>>>(in, in_re, tmp2, nt, nx, nx, 1, d_Wt, sign);
        dft_axis_kernel<<<nbk(n), 256, 0, s>>>(tmp2, nullptr, out, nx, nt, 1, nx, d_Wx, sign);
    };
    dft2(nullptr, acc_dev, spec, -1);
    dft2(nullptr, d_dat, specd, -1);
    static const double bands[3][2] = {{2.0, 3.5}, {3.5, 4.5}, {4.5, 6.0}};     // driver.f90:1812-1824
    std::vector<double> filt3((size_t)n);
    for (int b = 0; b < 3; ++b) {
        const std::vector<double> filt = freq_filter(bands[b][0], bands[b][1], nt, outputcad);
        for (int mode = 0; mode < 3; ++mode) {
            misfit[b * 3 + mode] = 0.0;
            nmeas[b * 3 + mode] = 0;
            if (!a.have_ridge[mode]) continue;
            const std::vector<double>& base = mode == 0 ? fm0 : pm0;
            for (int j = 0; j < nt; ++j)
                for (int i = 0; i < nx; ++i)
                    filt3[(size_t)j * nx + i] = (mode == 2 ? 1.0 : base[(size_t)j * nx + i]) * filt[j];
            cudaMemcpyAsync(d_filt, filt3.data(), n * 8, cudaMemcpyHostToDevice, s);
            spec_filter_kernel<<<nbk(n), 256, 0, s>>>(tmp, spec, d_filt, nullptr, nx, n);
            dft2(tmp, nullptr, A, +1);
            spec_filter_kernel<<<nbk(n), 256, 0, s>>>(tmp, specd, d_filt, nullptr, nx, n);
            dft2(tmp, nullptr, D, +1);
            RecvArgs ra;
            ra.nx = nx; ra.nt = nt; ra.mode = mode; ra.linesearch = (mode < 2 && a.linesearch) ? 1 : 0;
            ra.dt = a.dt; ra.t1 = a.t1; ra.x0 = a.x00; ra.xlength = xlength;
            ra.mindist = a.ridge[mode][0]; ra.maxdist = a.ridge[mode][1];
            ra.halftime = (int)std::floor(a.ridge[mode][2] / (2.0 * a.dt) + 0.5);
            ra.vel[0] = 1.01; ra.vel[1] = 1.465;                                  // driver.f90:1805-1806
            const double pc[5] = {r4(22.5000), r4(0.235317), r4(0.00134167), r4(-1.32222e-05), r4(3.00000e-08)};
            for (int q = 0; q < 5; ++q) ra.pc[q] = pc[q];                         // driver.f90:1909-1913
            ra.spectrum = 0;
            int* wb = windows + ((size_t)b * 2 + (mode < 2 ? mode : 0)) * 2 * nx;
            if (mode < 2) cudaMemcpyAsync(d_win, wb, 2 * nx * sizeof(int), cudaMemcpyHostToDevice, s);
            const size_t smc = (size_t)(2 * nt) * 8;
            if (smc > 48 * 1024) cudaFuncSetAttribute((const void*)receiver_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                      (int)smc);
            receiver_kernel<<<nx, 128, smc, s>>>(ra, A, D, nullptr, d_Wt, d_win, nullptr, d_tau, d_flag, d_err);
            std::vector<double> tau(nx);
            std::vector<int> flag(nx);
            cudaMemcpyAsync(tau.data(), d_tau, nx * 8, cudaMemcpyDeviceToHost, s);
            cudaMemcpyAsync(flag.data(), d_flag, nx * 4, cudaMemcpyDeviceToHost, s);
            if (mode < 2 && !a.linesearch)
                cudaMemcpyAsync(wb, d_win, 2 * nx * sizeof(int), cudaMemcpyDeviceToHost, s);
            if (cudaStreamSynchronize(s) != cudaSuccess) {
                why = std::string("CUDA error: ") + cudaGetErrorString(cudaGetLastError());
                return 2;
            }
            double sum = 0.0;
            for (int i = 0; i < nx; ++i)
                if (flag[i]) { sum = sum + std::pow(tau[i], 2.0); ++nmeas[b * 3 + mode]; }
            misfit[b * 3 + mode] = sum * 0.5;
        }
    }
    int herr = 0;
    cudaMemcpyAsync(&herr, d_err, 4, cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) {
        why = std::string("CUDA error: ") + cudaGetErrorString(cudaGetLastError());
        return 2;
    }
    if (herr) {
        why = herr == 1 ? "a measurement window starts or ends outside the record"
                        : (herr == 2 ? "a window [lef, rig] lies outside the record"
                                     : "a cross-correlation peak sits at the end of the lag range");
        return 1;
    }
    return 0;
}
