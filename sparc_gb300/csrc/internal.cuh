// Internal declarations shared by the CUDA translation units of libsparc_gpu.
//
// State representation.  For a background that depends on z only (the
// quiet-Sun cases of the reference), every operator of the time step --
// spectral x/y derivatives (derivatives.f90:28-170), the compact z derivative
// (dbyd2.f90), the PML (displacement.f90:495-560), spectral damping
// (damping.f90:125-161), the z and horizontal filters (physics.f90:741-833)
// and the point-wise equations -- acts independently on each horizontal
// Fourier mode (kx, ky).  The library therefore keeps the state as the 2-D
// r2c half-spectrum of every z-plane (normalised by 1/(nx*ny)) and advances
// each (kx, ky) z-pencil on its own.  Physical fields are produced only for
// outputs, by the shared-memory FFT kernels of fft.cu.
//
// Layout in HBM (T = double or float, CT = T2 complex):
//   spectral field:  [src][field][z][m],  m = ky*H + kx, H = nx/2+1, M = ny*H
//   physical field:  [z][y][x] (Fortran a(nx,ny,nz))
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>

template <typename T> struct CplxOf;
template <> struct CplxOf<double> { typedef double2 type; };
template <> struct CplxOf<float> { typedef float2 type; };

__host__ __device__ __forceinline__ double2 operator+(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ double2 operator-(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ double2 operator-(double2 a) { return make_double2(-a.x, -a.y); }
__host__ __device__ __forceinline__ double2 operator*(double s, double2 a) { return make_double2(s * a.x, s * a.y); }
__host__ __device__ __forceinline__ double2 operator*(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
__host__ __device__ __forceinline__ float2 operator+(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ float2 operator-(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ float2 operator-(float2 a) { return make_float2(-a.x, -a.y); }
__host__ __device__ __forceinline__ float2 operator*(float s, float2 a) { return make_float2(s * a.x, s * a.y); }
__host__ __device__ __forceinline__ float2 operator*(float2 a, float s) { return make_float2(a.x * s, a.y * s); }

template <typename CT> __host__ __device__ __forceinline__ CT czero();
template <> __host__ __device__ __forceinline__ double2 czero<double2>() { return make_double2(0.0, 0.0); }
template <> __host__ __device__ __forceinline__ float2 czero<float2>() { return make_float2(0.f, 0.f); }
template <typename V> __host__ __device__ __forceinline__ V vzero() { return V(0); }
template <> __host__ __device__ __forceinline__ double2 vzero<double2>() { return make_double2(0.0, 0.0); }
template <> __host__ __device__ __forceinline__ float2 vzero<float2>() { return make_float2(0.f, 0.f); }

// i*k*z for real k
template <typename T, typename CT>
__device__ __forceinline__ CT imul(T k, CT z) { CT r; r.x = -k * z.y; r.y = k * z.x; return r; }
// complex * complex
__device__ __forceinline__ double2 cmul(double2 a, double2 b) { return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) { return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }

// ---- z-profile table (T, nz entries per row) -------------------------------
enum ZTab {
    ZT_STRETCH = 0, ZT_UNSTRETCH, ZT_C2RHO0, ZT_GRADP0, ZT_RHO0, ZT_GRADRHO0, ZT_RHOINV, ZT_G,
    ZT_AZ, ZT_BZ, ZT_C2, ZT_GRAW,
    ZT_TH = 12,          // per bc b in 0..3: ZT_TH + 3*b + {0: lowr, 1: 1/betad, 2: gam}
    ZT_SRCDEP = ZT_TH + 12,   // source_dep (physics.f90:109), the velocity-form source profile
    ZT_COUNT
};
// ---- pencil table (T, M entries per row) ------------------------------------
enum PTab { PT_KX = 0, PT_KY, PT_DAMP, PT_HF, PT_COUNT };

// Compact-FD right-hand-side coefficients (dbyd2.f90:88-196), FP64 set-up
template <typename T> struct Compact {
    T C1, C2;          // interior (dbyd2.f90:88-89)
    T Cb[5];           // fourth-order near-boundary rows (dbyd2.f90:104-118)
    T Cf[4];           // fifth-order boundary rows (dbyd2.f90:122-146)
    T alpha2, beta1, cnst;   // boundary preconditioning (dbyd2.f90:157-173)
};

// Forward elimination of the compact-FD system for one pencil.
// ld(j) returns b(j) (0-based); bot/top are caller-set boundary values used
// for bc 2 (row 1) / bc 3 (row nz); y receives the eliminated values
// UD(J) = (R(J) - A(J) UD(J-1)) / BETAD(J)  (mtridag.f90:100-104).
template <typename V, typename T, typename Load>
__device__ __forceinline__ void compact_forward(int nz, int bc, Load ld, V bot, V top,
                                                const T* __restrict__ low, const T* __restrict__ ibd,
                                                const Compact<T>& c, V* y, long long ys) {
    V b0 = ld(0), b1 = ld(1), b2 = ld(2), b3 = ld(3), b4 = ld(4);
    V R1 = c.Cb[0] * b0 + c.Cb[1] * b1 + c.Cb[2] * b2 + c.Cb[3] * b3 + c.Cb[4] * b4;
    V R0;
    if (bc == 0) R0 = vzero<V>();
    else if (bc == 2) R0 = bot;
    else {
        R0 = c.Cf[0] * b0 + c.Cf[1] * b1 + c.Cf[2] * b2 + c.Cf[3] * b3;
        R0 = (c.alpha2 * R0 - c.beta1 * R1) * c.cnst;
    }
    V ud = R0 * __ldg(&ibd[0]);
    y[0] = ud;
    ud = (R1 - __ldg(&low[1]) * ud) * __ldg(&ibd[1]);
    y[ys] = ud;
    V w0 = b0, w1 = b1, w2 = b2, w3 = b3, w4 = b4;
    for (int j = 2; j <= nz - 3; ++j) {
        V R = c.C1 * (w3 - w1) + c.C2 * (w4 - w0);
        ud = (R - __ldg(&low[j]) * ud) * __ldg(&ibd[j]);
        y[(long long)j * ys] = ud;
        if (j + 3 <= nz - 1) { w0 = w1; w1 = w2; w2 = w3; w3 = w4; w4 = ld(j + 3); }
    }
    V Rn2 = -(c.Cb[0] * w4 + c.Cb[1] * w3 + c.Cb[2] * w2 + c.Cb[3] * w1 + c.Cb[4] * w0);
    V Rn1;
    if (bc == 0) Rn1 = vzero<V>();
    else if (bc == 3) Rn1 = top;
    else {
        Rn1 = -(c.Cf[0] * w4 + c.Cf[1] * w3 + c.Cf[2] * w2 + c.Cf[3] * w1);
        Rn1 = (c.alpha2 * Rn1 - c.beta1 * Rn2) * c.cnst;
    }
    ud = (Rn2 - __ldg(&low[nz - 2]) * ud) * __ldg(&ibd[nz - 2]);
    y[(long long)(nz - 2) * ys] = ud;
    ud = (Rn1 - __ldg(&low[nz - 1]) * ud) * __ldg(&ibd[nz - 1]);
    y[(long long)(nz - 1) * ys] = ud;
}

// z filter of FILTER_VARS_3D (physics.f90:758-786) / FILTER_VAR_Z
// (kernels.f90:845-881) / FILTER_VARS_2D (physics2d.f90:531-561) applied to a
// stream of values val(j); emit(j, filtered) is called for every j.
// mode 0: rows 2..nz-1 written (3-D);  mode 1: rows 6..nz-1 written (2-D, kst=6)
template <typename V, typename T, typename Load, typename Emit>
__device__ __forceinline__ void zfilter_stream(int nz, int mode, Load val, Emit emit) {
    const T h1 = (T)(0.5 * 0.41015625), h2 = (T)(0.5 * -0.234375), h3 = (T)(0.5 * 0.087890625);
    const T h4 = (T)(0.5 * -0.01953125), h5 = (T)(0.5 * 0.001953125), c0 = (T)0.75390625, hf = (T)0.5;
    // window w[q] = val(j - 5 + q)
    V w0 = vzero<V>(), w1 = vzero<V>(), w2 = vzero<V>(), w3 = vzero<V>(), w4 = vzero<V>();
    V w5 = val(0), w6 = val(1), w7 = val(2), w8 = val(3), w9 = val(4), w10 = val(5);
    for (int j = 0; j < nz; ++j) {
        V out;
        bool near_bot = (j >= 1 && j <= 4), near_top = (j >= nz - 5 && j <= nz - 2);
        if (j == 0 || j == nz - 1) out = w5;
        else if (near_top) out = hf * (w6 + w4);
        else if (near_bot) out = (mode == 0) ? hf * (w6 + w4) : w5;
        else
            out = c0 * w5 + h1 * (w4 + w6) + h2 * (w3 + w7) + h3 * (w2 + w8) + h4 * (w1 + w9) + h5 * (w0 + w10);
        emit(j, out);
        w0 = w1; w1 = w2; w2 = w3; w3 = w4; w4 = w5; w5 = w6; w6 = w7; w7 = w8; w8 = w9; w9 = w10;
        if (j + 6 < nz) w10 = val(j + 6);
    }
}

// ---- per-slot clocks (continuous batching) -------------------------------------
// Every source slot runs its own time index tl = time - t0[slot]: the source
// time series, LAGRANGE_INTERP, the horizontal-filter cadence and the output
// cadence all follow tl, so a request admitted into a free slot of a running
// batch starts at its own time 0 while sharing the batch's launches.
struct SlotClock {
    const int* t0;      // per-slot start (context time index at which the slot's clock read 0)
    const int* time;    // device counter: context time index of the step being taken
    int freq;           // freq_filtering (driver.f90:270)
    int two_d;          // option 17 cadence/gating rules
    int gate;           // forcing_length * cadforcing_step (driver.f90:421, physics2d.f90:1059)
    int num_steps;      // num_steps of LAGRANGE_INTERP (driver.f90:280-281)
    double ts, cad;     // timestep, cadforcing (REAL*4-rounded)
};

__device__ __forceinline__ bool slot_hfilter(const SlotClock& k, int tl) {
    // FILTER_VARS_3D: mod(time, freq) = 0 (physics.f90:791); FILTER_VARS_2D: mod(time+1, freq) = 0 (physics2d.f90:566)
    return tl >= 0 && (k.two_d ? ((tl + 1) % k.freq == 0) : (tl % k.freq == 0));
}
__device__ __forceinline__ bool slot_src_on(const SlotClock& k, int tl) {
    return tl >= 0 && (!k.two_d || tl <= k.gate);
}
// LAGRANGE_INTERP (physics.f90:683-734) at local time tl: the weights of
// vr(:,:,time1-3+l) (returned 0-based in idx), at most 7.  In 3-D the forcing
// is not re-interpolated after the gate (driver.f90:421-422), i.e. it keeps the
// value it had at the gate.
// One Lagrange weight l (0..6) of LAGRANGE_INTERP at local time tl: returns
// the weight and sets *id to the 0-based sample index, or returns 0 with
// *id = -1 when the sample l does not take part.
__device__ __forceinline__ double lagrange_weight(const SlotClock& k, int tl, int L, int l, int* id) {
    int t = tl;
    if (!k.two_d && t > k.gate) t = k.gate;
    double xt = (double)t * k.ts / k.cad;
    const int time1 = (int)floor(xt) + 1;
    xt = t * k.ts;
    const double Xl = (double)(time1 - 4 + l) * k.cad;
    const bool cond = (l <= 3) ? (Xl >= 0) : (l == 4 ? true : (l == 5 ? time1 < k.num_steps : time1 < k.num_steps - 1));
    const int i = time1 - 4 + l;
    *id = -1;
    if (!cond || i < 0 || i >= L) return 0.0;
    double den = 1.0, num = 1.0;
    #pragma unroll
    for (int r = 0; r < 7; ++r) {
        const double Xr = (double)(time1 - 4 + r) * k.cad;
        if (r != l) { den *= (Xl - Xr); num *= (xt - Xr); }
    }
    *id = i;
    return num / den;
}

// All weights, compacted: idx[0..n) and w[0..n).
__device__ __forceinline__ int lagrange_dev(const SlotClock& k, int tl, int L, int* idx, double* w) {
    int n = 0;
    #pragma unroll
    for (int l = 0; l < 7; ++l) {
        int id;
        const double wl = lagrange_weight(k, tl, L, l, &id);
        if (id < 0) continue;
        idx[n] = id;
        w[n] = wl;
        ++n;
    }
    return n;
}

// ---- register DFTs of the two-pass transforms (n = R*R) -----------------------
// W_n^q = exp(sign 2 pi i q / n) for 0 <= q < n from a table of n values
// (cos, sin of 2 pi q / n for q < n/2) in FP64, followed by the same n values
// in FP32 (read by the FP32 kernels, so no conversion on the FP64 pipe)
template <typename T> __device__ __forceinline__ T tw_val(const double* __restrict__ tw, int n, int i);
template <> __device__ __forceinline__ double tw_val<double>(const double* __restrict__ tw, int, int i) {
    return __ldg(&tw[i]);
}
template <> __device__ __forceinline__ float tw_val<float>(const double* __restrict__ tw, int n, int i) {
    return __ldg(&reinterpret_cast<const float*>(tw + n)[i]);
}
template <typename T, typename CT>
__device__ __forceinline__ CT tw_n(const double* __restrict__ tw, int q, int n, T sign) {
    const int h = n >> 1;
    const bool flip = q >= h;
    const int r = flip ? q - h : q;
    T c = tw_val<T>(tw, n, 2 * r), sn = sign * tw_val<T>(tw, n, 2 * r + 1);
    if (flip) { c = -c; sn = -sn; }
    CT w;
    w.x = c;
    w.y = sn;
    return w;
}

// Paired FP32 arithmetic (FFMA2 / FADD2 / FMUL2, sm_100 and later): one
// instruction for both components of a float2 (the two parts of a complex
// value, or two neighbouring pencils).  bc2 broadcasts a multiplier shared by
// both components; psub is an FFMA2 with -1, which rounds exactly as the
// subtraction.
__device__ __forceinline__ float2 bc2(float s) { return make_float2(s, s); }
__device__ __forceinline__ float2 pfma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 pmul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 padd(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 psub(float2 a, float2 b) { return __ffma2_rn(make_float2(-1.f, -1.f), b, a); }

// butterfly sum and difference; in FP32 one paired instruction each (FADD2,
// and FFMA2 with -1, which rounds exactly as the subtraction)
__device__ __forceinline__ double2 bsum(double2 a, double2 c) { return a + c; }
__device__ __forceinline__ double2 bdif(double2 a, double2 c) { return make_double2(a.x - c.x, a.y - c.y); }
#if defined(__CUDA_ARCH__)
__device__ __forceinline__ float2 bsum(float2 a, float2 c) { return __fadd2_rn(a, c); }
__device__ __forceinline__ float2 bdif(float2 a, float2 c) { return __ffma2_rn(make_float2(-1.f, -1.f), c, a); }
#else
__device__ __forceinline__ float2 bsum(float2 a, float2 c) { return a + c; }
__device__ __forceinline__ float2 bdif(float2 a, float2 c) { return make_float2(a.x - c.x, a.y - c.y); }
#endif

// in-register DFT of length R (decimation in frequency): on return v[brev(k)]
// holds X[k]; w[j] = W_R^j for j < R/2
template <typename CT, int R>
__device__ __forceinline__ void reg_dft(CT (&v)[R], const CT (&w)[R / 2]) {
    #pragma unroll
    for (int len = R; len >= 2; len >>= 1) {
        const int half = len >> 1, step = R / len;
        #pragma unroll
        for (int b = 0; b < R; b += len) {
            #pragma unroll
            for (int k = 0; k < half; ++k) {
                const CT a = v[b + k], c = v[b + k + half];
                v[b + k] = bsum(a, c);
                const CT d = bdif(a, c);
                v[b + k + half] = (k == 0) ? d : cmul(d, w[k * step]);
            }
        }
    }
}

template <int R>
__host__ __device__ constexpr int brev(int k) {
    int r = 0;
    for (int b = 1, m = R >> 1; b < R; b <<= 1, m >>= 1)
        if (k & b) r |= m;
    return r;
}


// Stockham radix-2 over `count` sequences of length n stored back to back in
// src; returns the buffer that holds the result.  tw[2q], tw[2q+1] =
// cos, sin(2 pi q / n) for q < n/2 (the twiddle table of tw_val, computed on the host).
template <typename T, typename CT>
__device__ __forceinline__ CT* smem_fft(CT* src, CT* dst, int n, int count, T sign, const double* __restrict__ tw) {
    const int half = n >> 1;
    const int total = half * count;
    for (int Ns = 1; Ns < n; Ns <<= 1) {
        const int stride = n / (2 * Ns);
        for (int t = threadIdx.x; t < total; t += blockDim.x) {
            const int seq = t / half, j = t - seq * half;
            CT* s = src + seq * n;
            CT* d = dst + seq * n;
            const int k = j & (Ns - 1);
            CT v0 = s[j], v1 = s[j + half];
            const int q = k * stride;
            const T c = tw_val<T>(tw, n, 2 * q);
            const T sn = sign * tw_val<T>(tw, n, 2 * q + 1);
            CT w;
            w.x = v1.x * c - v1.y * sn;
            w.y = v1.x * sn + v1.y * c;
            const int idx = ((j - k) << 1) + k;
            d[idx] = v0 + w;
            d[idx + Ns] = v0 - w;
        }
        __syncthreads();
        CT* tmp = src; src = dst; dst = tmp;
    }
    return src;
}

// ---- argument blocks ----------------------------------------------------------
template <typename T> struct StageArgs {
    typedef typename CplxOf<T>::type CT;
    CT* a; CT* scr; CT* pml; CT* scrpml; CT* ybuf; CT* pbuf; CT* rbuf;
    const T* zt; const T* pt;
    long long fs;       // spectral field stride nz*M
    long long ps;       // pml field stride nzpml*M
    int M, nz, npmlbot, npmltop, option, damp;
    int has_scr;
    int block;          // threads per CTA (64 or 128; same results, a tuning choice)
    int q, chunk;       // lanes per pencil (1, 2, 4, 8) and levels per lane (stage_chunk_kernel)
    const T* zc;        // its products of the elimination multipliers: H, G of the xi_z code, H, G of the p' code
    T beta;
    Compact<T> cc;
    // source injection at plane ksrc (0-based)
    int src_mode, ksrc;         // 0 none, 1 series, 2 Lagrange
    T src_scale;                // delta_width / rho0(ksrc)
    const CT* planes; long long plane_ss; int L;
    const double* series; int nseries;
    SlotClock clk;
};

template <typename T> struct UpdateArgs {
    typedef typename CplxOf<T>::type CT;
    CT* a; CT* scr; CT* pml; CT* scrpml;
    const T* pt;
    long long fs, ps;
    int M, nz, nzpml, option;
    T dt;
    SlotClock clk;      // the horizontal filter follows each slot's clock
    int block;          // threads per CTA (32, 64 or 128), as the stage kernels
    int q, chunk;       // lanes per pencil and levels per lane, as the stage kernels
    CT* ybuf;           // per-source scratch column (the chunked form's staging)
};

// fused FP32 step (fused.cu)
// z table of the fused FP32 step, [FZ_COUNT][NZP] (NZP = fused_nzp(nz), padded
// rows zero): profile rows, then the five elimination rows (1/betad,
// elimination multiplier m, the carry response K = H + g K(next) of the
// chunk's back substitution, H the chunk products of m, back-substitution
// multiplier g, chunk products G of g) of the xi_z boundary code and of the p'
// boundary code, then the look-back products of each code: a forward row and
// a backward row, [chunk t][4] floats each (the products of the multipliers
// of the 1..4 chunks between chunk t and the chunk 2..5 below / above it).
// The elimination rows solve for s(j) x(j) instead of x(j), s = stretch for
// xi_z and stretch / rho0 for p' (the factors the step applies to the two
// derivatives): 1/betad and the multipliers carry the ratios of s, so the
// solves return the scaled derivatives directly.
enum {
    FZ_AZR = 0, FZ_C2R, FZ_GP, FZ_RI, FZ_E1, FZ_E2, FZ_AZ, FZ_BZ, FZ_SX = 8, FZ_SP = 13,
    FZ_LX = 18, FZ_LP = 20, FZ_COUNT = 22
};
constexpr int FUSED_KB = 5;    // chunks summed by a look-back carry of the fused step
// largest product of chunk multipliers over FUSED_KB chunks (the first term a
// look-back carry leaves out) for which the fused step is used
constexpr double FUSED_LOOKBACK_BOUND = 2.3283064365386963e-10;   // 2^-32
struct FusedArgs {
    float2* a; float2* scr; float2* pml;
    const float* ftab; const float* pt;
    float unstr_top;
    long long fs, ps;
    int M, nz, nzpml, npmlbot, npmltop, option, damp, W;
    float betas[5];
    float dt;
    Compact<float> cc;
    int write_scr;
    int src_mode, ksrc;
    float src_scale;
    const float2* planes; long long plane_ss; int L;
    const double* series; int nseries;
    SlotClock clk;
    int pencils;        // modes per CTA: 2, 4 or 8 (same results; a tuning choice)
    int* err;           // set to 1 if the bounded wait for the z-table bulk copy gave up
    int wait_limit;     // polls of that wait before it gives up
    int no_copy;        // test switch: issue no bulk copy, so the wait runs out with nothing in flight
    float2* src_plane;  // [S][M] this step's interpolated source plane (src_mode 2, source_plane_kernel)
    int nsrc;           // sources of the launch (set by the launcher)
    int pf_stride;      // > 0: each CTA prefetches into L2 the rows of the CTA pf_stride later in launch
                        // order (set by the launcher to the CTAs resident at once); 0: no prefetch
};
constexpr int FUSED_CH = 5;
void fused_prepare(int nz, int nzpml);
size_t fused_smem_bytes(int nz, int nzpml, int W);
bool fused_fits(int P, int nz, int nzpml);
int fused_supported(int nz);
int fused_w(int nz);
int fused_nzp(int nz);
void launch_fused(const FusedArgs& A, int nsrc, cudaStream_t s);
void launch_source_plane(const FusedArgs& A, int nsrc, cudaStream_t s);

// launchers (modal.cu)
template <typename T> void launch_stage(const StageArgs<T>& A, int nsrc, cudaStream_t s);
template <typename T> void launch_update(const UpdateArgs<T>& A, int nsrc, cudaStream_t s);
// surface record of field `field` (v_z) at plane kplane for every slot whose clock is on the output cadence
template <typename T>
void launch_record(const typename CplxOf<T>::type* a, typename CplxOf<T>::type* rec, const int* t0, const int* time,
                   int steps, int rec_max, long long fs, int M, int kplane, int field, int nsrc, cudaStream_t s);
// the device time counter: set, and advance by one step
void launch_set_time(int* time, int value, cudaStream_t s);
void launch_tick(int* time, cudaStream_t s);
template <typename T>
void launch_zderiv(const T* zt, const Compact<T>& cc, const typename CplxOf<T>::type* in,
                   typename CplxOf<T>::type* out, long long n1, int nz, int bc, int filter,
                   const typename CplxOf<T>::type* top_plane, int nsrc, long long in_ss, long long out_ss,
                   cudaStream_t s);
void launch_zderiv_real(const double* zt, const Compact<double>& cc, const double* in, double* out,
                        long long n1, int nz, int bc, cudaStream_t s);

// geometry of a context for the no-allocation transform (noalloc.cu)
#define SPARC_NOALLOC_SCRATCH_BYTES (32u << 20)
struct sparc_ctx;
struct SparcXformInfo {
    int nx, ny, M, f32;
    const double* tw_x;
    const double* tw_y;
    cudaStream_t stream;
};
__attribute__((visibility("hidden"))) void sparc_internal_xform_info(const sparc_ctx* c, SparcXformInfo* out);
__attribute__((visibility("hidden"))) void sparc_internal_set_error(sparc_ctx* c, const std::string& msg);
__attribute__((visibility("hidden"))) void sparc_internal_count_launches(sparc_ctx* c, int n);

// transforms (fft.cu)
template <typename T>
void fft_phys_to_spec(const T* phys, typename CplxOf<T>::type* spec, typename CplxOf<T>::type* tmp,
                      int nx, int ny, int nplanes, const double* tw_x, const double* tw_y, cudaStream_t s,
                      const T* mul = nullptr);
template <typename T>
void fft_spec_to_phys(const typename CplxOf<T>::type* spec, T* phys, typename CplxOf<T>::type* tmp,
                      int nx, int ny, int nplanes, const double* tw_x, const double* tw_y, cudaStream_t s);
// phys -> out through the spectrum times the real multiplier mul[ky][kx];
// returns the number of launches
template <typename T>
int fft_filter_phys(const T* phys, T* out, typename CplxOf<T>::type* spec, typename CplxOf<T>::type* tmp, int nx,
                    int ny, int nplanes, const double* tw_x, const double* tw_y, cudaStream_t s, const T* mul);
// the same with grouped input planes: plane p of the input starts at
// spec + (p / ppg) * gstride + (p % ppg) * ny * (nx/2+1) (complex elements);
// phys and tmp are contiguous
template <typename T>
void fft_spec_to_phys_g(const typename CplxOf<T>::type* spec, int ppg, long long gstride, T* phys,
                        typename CplxOf<T>::type* tmp, int nx, int ny, int nplanes, const double* tw_x,
                        const double* tw_y, cudaStream_t s);

// kernel (sensitivity) helpers (fft.cu)
// (nsrc sources on grid.y; out_ss / in_ss: per-source strides in elements)
template <typename T>
void launch_spec_combine(typename CplxOf<T>::type* out, const typename CplxOf<T>::type* fx,
                         const typename CplxOf<T>::type* fy, const T* pt, int M, int nz, int nsrc, long long out_ss,
                         long long in_ss, cudaStream_t s);
template <typename T>
void launch_spec_scale_z(typename CplxOf<T>::type* out, const typename CplxOf<T>::type* in,
                         const T* zt, int row, int M, int nz, int nsrc, long long out_ss, long long in_ss,
                         cudaStream_t s);
template <typename T>
void launch_spec_dxdy(typename CplxOf<T>::type* out, const typename CplxOf<T>::type* in,
                      const T* pt, int which, int M, int nz, int nsrc, long long out_ss, long long in_ss,
                      cudaStream_t s);
// acc [nsrc][3][N]; fwd field f of source g at fwd + f*fwd_fs + g*N, adj likewise
template <typename T>
// c2f: per-point c^2 (a 2-D background) instead of the z profile, or null
void launch_kernel_accum(double* acc, const T* fwd, long long fwd_fs, const T* adj, long long adj_fs,
                         const double* zt64, long long NP, int nz, int use_y, int nsrc, cudaStream_t s,
                         const double* c2f = nullptr);
template <typename T>
void launch_copy_convert(T* dst, const double* src, long long n, cudaStream_t s);
template <typename T>
void launch_copy_back(double* dst, const T* src, long long n, cudaStream_t s);
void launch_spec_mult(double2* spec, const double* mult, long long M, int nplanes, cudaStream_t s);
int launch_check_finite_f64(const double* p, long long n, int* flag, cudaStream_t s);
int launch_check_finite_f32(const float* p, long long n, int* flag, cudaStream_t s);
void launch_kernel_finish(double* out, const double* acc, const double* zt64, long long NP, int nz,
                          double scale_c, double scale_r, int nsum, long long acc_ss, cudaStream_t s,
                          const double* r0f = nullptr, const double* c2f = nullptr);
