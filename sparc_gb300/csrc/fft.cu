// Horizontal transforms between physical planes a(nx,ny) and the normalised
// r2c half-spectrum state, written as shared-memory Stockham radix-2 FFTs
// (the FFTW plans of initialize.f90:323-337 and damping.f90:46-58 are the
// reference's counterpart; cuFFT is not used).
//
//   phys -> spec : rows_r2c   (two real rows packed as one complex FFT along x,
//                              split by Hermitian symmetry, scaled 1/(nx*ny))
//                  cols_fft   (complex FFT along y on tiles of kx columns)
//   spec -> phys : cols_fft (inverse), rows_c2r (two rows per complex inverse
//                  FFT; DC/Nyquist imaginary parts dropped as FFTW c2r does)
//
// Also: point-wise spectral multipliers and the sensitivity-kernel
// accumulation of kernels.f90:273-311 on physical fields.
#include "internal.cuh"

// offset of input plane p when planes come in groups of ppg, group g starting
// at g * gstride (complex elements); pe = elements per plane
__device__ __forceinline__ long long grp_off(long long p, int ppg, long long gstride, long long pe) {
    const long long g = p / ppg;
    return g * gstride + (p - g * ppg) * pe;
}

// phys (nrows rows of nx reals) -> out (nrows rows of H = nx/2+1 complex), scaled by `scale`
template <typename T>
__global__ void rows_r2c_kernel(const T* __restrict__ phys, typename CplxOf<T>::type* __restrict__ out,
                                int nx, long long nrows, T scale, const double* __restrict__ tw) {
    typedef typename CplxOf<T>::type CT;
    extern __shared__ __align__(16) unsigned char smraw[];
    CT* b0 = (CT*)smraw;
    CT* b1 = b0 + nx;
    const long long r0 = 2LL * blockIdx.x, r1 = r0 + 1;
    const bool has1 = r1 < nrows;
    for (int i = threadIdx.x; i < nx; i += blockDim.x) {
        CT v;
        v.x = phys[r0 * nx + i];
        v.y = has1 ? phys[r1 * nx + i] : (T)0;
        b0[i] = v;
    }
    __syncthreads();
    CT* Z = smem_fft<T, CT>(b0, b1, nx, 1, (T)-1, tw);
    const int H = nx / 2 + 1;
    const T hs = (T)0.5 * scale;
    for (int k = threadIdx.x; k < H; k += blockDim.x) {
        CT zk = Z[k], zn = Z[(nx - k) & (nx - 1)];
        CT x1, x2;
        x1.x = (zk.x + zn.x) * hs;
        x1.y = (zk.y - zn.y) * hs;
        x2.x = (zk.y + zn.y) * hs;
        x2.y = -(zk.x - zn.x) * hs;
        out[r0 * H + k] = x1;
        if (has1) out[r1 * H + k] = x2;
    }
}

// in (nrows rows of H complex) -> phys (nrows rows of nx reals), inverse, unscaled
template <typename T>
__global__ void rows_c2r_kernel(const typename CplxOf<T>::type* __restrict__ in, T* __restrict__ phys,
                                int nx, long long nrows, const double* __restrict__ tw, int ny, int ppg,
                                long long gstride) {
    typedef typename CplxOf<T>::type CT;
    extern __shared__ __align__(16) unsigned char smraw[];
    CT* b0 = (CT*)smraw;
    CT* b1 = b0 + nx;
    const long long r0 = 2LL * blockIdx.x, r1 = r0 + 1;
    const bool has1 = r1 < nrows;
    const int H = nx / 2 + 1, half = nx / 2;
    const long long pe = (long long)ny * H;
    const long long o0 = grp_off(r0 / ny, ppg, gstride, pe) + (r0 % ny) * H;
    const long long o1 = has1 ? grp_off(r1 / ny, ppg, gstride, pe) + (r1 % ny) * H : 0;
    for (int k = threadIdx.x; k <= half; k += blockDim.x) {
        CT x1 = in[o0 + k];
        CT x2 = has1 ? in[o1 + k] : czero<CT>();
        if (k == 0 || k == half) {
            CT z; z.x = x1.x; z.y = x2.x;
            b0[k] = z;
        } else {
            CT z;
            z.x = x1.x - x2.y; z.y = x1.y + x2.x;
            b0[k] = z;
            z.x = x1.x + x2.y; z.y = -x1.y + x2.x;
            b0[nx - k] = z;
        }
    }
    __syncthreads();
    CT* Z = smem_fft<T, CT>(b0, b1, nx, 1, (T)1, tw);
    for (int i = threadIdx.x; i < nx; i += blockDim.x) {
        CT z = Z[i];
        phys[r0 * nx + i] = z.x;
        if (has1) phys[r1 * nx + i] = z.y;
    }
}

// complex FFT along y on tiles of W kx-columns: data [plane][y][kx], H columns
template <typename T>
__global__ void cols_fft_kernel(const typename CplxOf<T>::type* __restrict__ in,
                                typename CplxOf<T>::type* __restrict__ out, int ny, int H, int W, T sign,
                                const double* __restrict__ tw, int ppg, long long gstride) {
    typedef typename CplxOf<T>::type CT;
    extern __shared__ __align__(16) unsigned char smraw[];
    CT* b0 = (CT*)smraw;
    CT* b1 = b0 + (long long)W * ny;
    const int ntile = (H + W - 1) / W;
    const long long plane = blockIdx.x / ntile;
    const int kx0 = (blockIdx.x % ntile) * W;
    const int w = min(W, H - kx0);
    const long long base = plane * (long long)ny * H;
    const long long ibase = grp_off(plane, ppg, gstride, (long long)ny * H);
    for (int t = threadIdx.x; t < W * ny; t += blockDim.x) {
        int y = t / W, c = t - y * W;
        b0[c * ny + y] = (c < w) ? in[ibase + (long long)y * H + kx0 + c] : czero<CT>();
    }
    __syncthreads();
    CT* Z = smem_fft<T, CT>(b0, b1, ny, W, sign, tw);
    for (int t = threadIdx.x; t < W * ny; t += blockDim.x) {
        int y = t / W, c = t - y * W;
        if (c < w) out[base + (long long)y * H + kx0 + c] = Z[c * ny + y];
    }
}

// ---- two-pass transforms for n = R*R (R = 8, 16): n = R*n1 + n2,
// k = k1 + R*k2.  Pass 1 (thread n2): R-point DFT over n1 of x[R n1 + n2],
// times the twiddle W_n^(n2 k1); pass 2 (thread k1): R-point DFT over n2.
// Each DFT runs in registers; one shared-memory exchange and one barrier per
// CTA.  W_m^j = exp(sign 2 pi i j / m) comes from the FP64 table tw
// (cos, sin of 2 pi q / n for q < n/2).

// complex FFT along y (length ny = R*R) for NC = 256/R kx-columns per CTA;
// data [plane][y][kx] with H columns per row
template <typename T, int R>
__global__ void __launch_bounds__(256) cols_fft_sq_kernel(const typename CplxOf<T>::type* __restrict__ in,
                                                          typename CplxOf<T>::type* __restrict__ out, int H,
                                                          T sign, const double* __restrict__ tw, int ppg,
                                                          long long gstride, const T* __restrict__ mul) {
    typedef typename CplxOf<T>::type CT;
    constexpr int n = R * R, NC = 256 / R;
    extern __shared__ __align__(16) unsigned char smraw[];
    CT* Z = (CT*)smraw;                                  // [k1][n2][c]
    const int ntile = (H + NC - 1) / NC;
    const long long plane = blockIdx.x / ntile;
    const int kx0 = (blockIdx.x % ntile) * NC;
    const int c = threadIdx.x % NC, r = threadIdx.x / NC;
    const bool cv = kx0 + c < H;
    const long long base = plane * (long long)n * H + kx0 + c;
    const long long ibase = grp_off(plane, ppg, gstride, (long long)n * H) + kx0 + c;
    CT w[R / 2];
    #pragma unroll
    for (int j = 0; j < R / 2; ++j) w[j] = tw_n<T, CT>(tw, j * R, n, sign);
    // pass 1: thread n2 = r
    CT v[R];
    #pragma unroll
    for (int n1 = 0; n1 < R; ++n1) v[n1] = cv ? in[ibase + (long long)(R * n1 + r) * H] : czero<CT>();
    reg_dft<CT, R>(v, w);
    #pragma unroll
    for (int k1 = 0; k1 < R; ++k1) {
        CT y = v[brev<R>(k1)];
        if (k1 > 0 && r > 0) y = cmul(y, tw_n<T, CT>(tw, r * k1, n, sign));
        Z[(k1 * R + r) * NC + c] = y;
    }
    __syncthreads();
    // pass 2: thread k1 = r
    #pragma unroll
    for (int n2 = 0; n2 < R; ++n2) v[n2] = Z[(r * R + n2) * NC + c];
    reg_dft<CT, R>(v, w);
    if (cv) {
        #pragma unroll
        for (int k2 = 0; k2 < R; ++k2) {
            CT val = v[brev<R>(k2)];
            if (mul) val = __ldg(&mul[(long long)(r + R * k2) * H + kx0 + c]) * val;   // a real pencil multiplier
            out[base + (long long)(r + R * k2) * H] = val;
        }
    }
}

// cols_fft_sq_kernel forward, the real multiplier mul[ky][kx], and
// cols_fft_sq_kernel inverse in one pass, in place on [plane][y][kx] columns:
// after the forward passes thread r holds the indices r + R k2, which are the
// ones the inverse's first pass loads, so both halves are the standalone
// kernels' arithmetic and the result equals the two-kernel path bit for bit
template <typename T, int R>
__global__ void __launch_bounds__(256) cols_filter_sq_kernel(typename CplxOf<T>::type* __restrict__ data, int H,
                                                             const double* __restrict__ tw,
                                                             const T* __restrict__ mul) {
    typedef typename CplxOf<T>::type CT;
    constexpr int n = R * R, NC = 256 / R;
    extern __shared__ __align__(16) unsigned char smraw[];
    CT* Z = (CT*)smraw;                                  // [k1][n2][c]
    const int ntile = (H + NC - 1) / NC;
    const long long plane = blockIdx.x / ntile;
    const int kx0 = (blockIdx.x % ntile) * NC;
    const int c = threadIdx.x % NC, r = threadIdx.x / NC;
    const bool cv = kx0 + c < H;
    const long long base = plane * (long long)n * H + kx0 + c;
    CT wf[R / 2], wi[R / 2];
    #pragma unroll
    for (int j = 0; j < R / 2; ++j) {
        wf[j] = tw_n<T, CT>(tw, j * R, n, (T)-1);
        wi[j] = tw_n<T, CT>(tw, j * R, n, (T)1);
    }
    CT v[R];
    #pragma unroll
    for (int n1 = 0; n1 < R; ++n1) v[n1] = cv ? data[base + (long long)(R * n1 + r) * H] : czero<CT>();
    // forward, pass 1 (thread n2 = r) and pass 2 (thread k1 = r)
    reg_dft<CT, R>(v, wf);
    #pragma unroll
    for (int k1 = 0; k1 < R; ++k1) {
        CT y = v[brev<R>(k1)];
        if (k1 > 0 && r > 0) y = cmul(y, tw_n<T, CT>(tw, r * k1, n, (T)-1));
        Z[(k1 * R + r) * NC + c] = y;
    }
    __syncthreads();
    #pragma unroll
    for (int n2 = 0; n2 < R; ++n2) v[n2] = Z[(r * R + n2) * NC + c];
    reg_dft<CT, R>(v, wf);
    CT u[R];
    #pragma unroll
    for (int k2 = 0; k2 < R; ++k2) {
        const CT X = v[brev<R>(k2)];
        u[k2] = cv ? __ldg(&mul[(long long)(r + R * k2) * H + kx0 + c]) * X : czero<CT>();
    }
    __syncthreads();                                     // every thread has read its forward tile
    // inverse, pass 1 (thread n2 = r holds indices R n1 + r) and pass 2
    reg_dft<CT, R>(u, wi);
    #pragma unroll
    for (int k1 = 0; k1 < R; ++k1) {
        CT y = u[brev<R>(k1)];
        if (k1 > 0 && r > 0) y = cmul(y, tw_n<T, CT>(tw, r * k1, n, (T)1));
        Z[(k1 * R + r) * NC + c] = y;
    }
    __syncthreads();
    #pragma unroll
    for (int n2 = 0; n2 < R; ++n2) u[n2] = Z[(r * R + n2) * NC + c];
    reg_dft<CT, R>(u, wi);
    if (cv) {
        #pragma unroll
        for (int k2 = 0; k2 < R; ++k2) data[base + (long long)(r + R * k2) * H] = u[brev<R>(k2)];
    }
}

// inverse real transform along x (length nx = R*R), two rows per complex
// FFT as rows_c2r_kernel, NP = 256/R row pairs per CTA
template <typename T, int R>
__global__ void __launch_bounds__(256) rows_c2r_sq_kernel(const typename CplxOf<T>::type* __restrict__ in,
                                                          T* __restrict__ phys, long long nrows,
                                                          const double* __restrict__ tw, int ny, int ppg,
                                                          long long gstride) {
    typedef typename CplxOf<T>::type CT;
    constexpr int nx = R * R, H = nx / 2 + 1, half = nx / 2, NP = 256 / R;
    extern __shared__ __align__(16) unsigned char smraw[];
    CT* Z = (CT*)smraw;                                  // [pair][k1][R+1]
    const int r = threadIdx.x % R, pp = threadIdx.x / R;
    const long long r0 = 2LL * ((long long)blockIdx.x * NP + pp), r1 = r0 + 1;
    const bool has0 = r0 < nrows, has1 = r1 < nrows;
    const long long pe = (long long)ny * H;
    const long long o0 = has0 ? grp_off(r0 / ny, ppg, gstride, pe) + (r0 % ny) * H : 0;
    const long long o1 = has1 ? grp_off(r1 / ny, ppg, gstride, pe) + (r1 % ny) * H : 0;
    CT w[R / 2];
    #pragma unroll
    for (int j = 0; j < R / 2; ++j) w[j] = tw_n<T, CT>(tw, j * R, nx, (T)1);
    // pass 1: thread n2 = r gathers z[R n1 + n2] of the packed pair
    CT v[R];
    #pragma unroll
    for (int n1 = 0; n1 < R; ++n1) {
        const int idx = R * n1 + r;
        const bool mirror = idx > half;
        const int k = mirror ? nx - idx : idx;
        const CT x1 = has0 ? in[o0 + k] : czero<CT>();
        const CT x2 = has1 ? in[o1 + k] : czero<CT>();
        CT z;
        if (k == 0 || k == half) { z.x = x1.x; z.y = x2.x; }
        else if (!mirror) { z.x = x1.x - x2.y; z.y = x1.y + x2.x; }
        else { z.x = x1.x + x2.y; z.y = -x1.y + x2.x; }
        v[n1] = z;
    }
    reg_dft<CT, R>(v, w);
    CT* Zp = Z + pp * R * (R + 1);
    #pragma unroll
    for (int k1 = 0; k1 < R; ++k1) {
        CT y = v[brev<R>(k1)];
        if (k1 > 0 && r > 0) y = cmul(y, tw_n<T, CT>(tw, r * k1, nx, (T)1));
        Zp[k1 * (R + 1) + r] = y;
    }
    __syncthreads();
    // pass 2: thread k1 = r
    #pragma unroll
    for (int n2 = 0; n2 < R; ++n2) v[n2] = Zp[r * (R + 1) + n2];
    reg_dft<CT, R>(v, w);
    #pragma unroll
    for (int k2 = 0; k2 < R; ++k2) {
        const CT zz = v[brev<R>(k2)];
        if (has0) phys[r0 * nx + r + R * k2] = zz.x;
        if (has1) phys[r1 * nx + r + R * k2] = zz.y;
    }
}

// forward real transform along x (length nx = R*R) of two rows packed as one
// complex FFT, split by Hermitian symmetry and scaled as rows_r2c_kernel;
// NP = 256/R row pairs per CTA
template <typename T, int R>
__global__ void __launch_bounds__(256) rows_r2c_sq_kernel(const T* __restrict__ phys,
                                                          typename CplxOf<T>::type* __restrict__ out,
                                                          long long nrows, T scale, const double* __restrict__ tw) {
    typedef typename CplxOf<T>::type CT;
    constexpr int nx = R * R, H = nx / 2 + 1, NP = 256 / R;
    extern __shared__ __align__(16) unsigned char smraw[];
    const int r = threadIdx.x % R, pp = threadIdx.x / R;
    CT* Zp = (CT*)smraw + pp * R * (R + 1);              // [k1][R+1], then the spectrum [k]
    const long long r0 = 2LL * ((long long)blockIdx.x * NP + pp), r1 = r0 + 1;
    const bool has0 = r0 < nrows, has1 = r1 < nrows;
    CT w[R / 2];
    #pragma unroll
    for (int j = 0; j < R / 2; ++j) w[j] = tw_n<T, CT>(tw, j * R, nx, (T)-1);
    CT v[R];
    #pragma unroll
    for (int n1 = 0; n1 < R; ++n1) {
        v[n1].x = has0 ? phys[r0 * nx + R * n1 + r] : (T)0;
        v[n1].y = has1 ? phys[r1 * nx + R * n1 + r] : (T)0;
    }
    reg_dft<CT, R>(v, w);
    #pragma unroll
    for (int k1 = 0; k1 < R; ++k1) {
        CT y = v[brev<R>(k1)];
        if (k1 > 0 && r > 0) y = cmul(y, tw_n<T, CT>(tw, r * k1, nx, (T)-1));
        Zp[k1 * (R + 1) + r] = y;
    }
    __syncthreads();
    #pragma unroll
    for (int n2 = 0; n2 < R; ++n2) v[n2] = Zp[r * (R + 1) + n2];
    reg_dft<CT, R>(v, w);
    __syncthreads();                                     // the tile now takes the spectrum
    #pragma unroll
    for (int k2 = 0; k2 < R; ++k2) Zp[r + R * k2] = v[brev<R>(k2)];
    __syncthreads();
    const T hs = (T)0.5 * scale;
    for (int k = r; k < H; k += R) {
        const CT zk = Zp[k], zn = Zp[(nx - k) & (nx - 1)];
        CT x1, x2;
        x1.x = (zk.x + zn.x) * hs;
        x1.y = (zk.y - zn.y) * hs;
        x2.x = (zk.y + zn.y) * hs;
        x2.y = -(zk.x - zn.x) * hs;
        if (has0) out[r0 * H + k] = x1;
        if (has1) out[r1 * H + k] = x2;
    }
}

static int sq_radix(int n) { return n == 256 ? 16 : (n == 64 ? 8 : 0); }

static int col_tile(int ny) { return ny >= 1024 ? 4 : (ny >= 512 ? 8 : 16); }

template <typename T>
static void set_smem(const void* fn, size_t bytes) {
    static size_t done = 0;
    (void)done;
    cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

// spec[plane][m] *= mul[m] (a real pencil multiplier, m < M)
template <typename T>
__global__ void spec_mul_kernel(typename CplxOf<T>::type* spec, const T* __restrict__ mul, int M, long long n) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) spec[t] = mul[t % M] * spec[t];
}

// phys -> normalised half-spectrum; with mul, each spectral plane is also
// multiplied by the real pencil multiplier mul[m] (in the column pass when
// there is one)
// rows of nx reals -> rows of H complex (the forward row pass of fft_phys_to_spec)
template <typename T>
static void rows_forward(const T* phys, typename CplxOf<T>::type* dst, int nx, long long nrows, T scale,
                         const double* tw_x, cudaStream_t s) {
    typedef typename CplxOf<T>::type CT;
    const int Rx = sq_radix(nx);
    if (Rx) {
        const long long rows_per_cta = 2LL * (256 / Rx);
        const unsigned grid = (unsigned)((nrows + rows_per_cta - 1) / rows_per_cta);
        const size_t smr = (size_t)(256 / Rx) * Rx * (Rx + 1) * sizeof(CT);
        if (Rx == 16) {
            set_smem<T>((const void*)rows_r2c_sq_kernel<T, 16>, smr);
            rows_r2c_sq_kernel<T, 16><<<grid, 256, smr, s>>>(phys, dst, nrows, scale, tw_x);
        } else {
            set_smem<T>((const void*)rows_r2c_sq_kernel<T, 8>, smr);
            rows_r2c_sq_kernel<T, 8><<<grid, 256, smr, s>>>(phys, dst, nrows, scale, tw_x);
        }
    } else {
        size_t sm = 2 * (size_t)nx * sizeof(CT);
        int thr = nx / 2 < 256 ? (nx / 2 < 32 ? 32 : nx / 2) : 256;
        set_smem<T>((const void*)rows_r2c_kernel<T>, sm);
        rows_r2c_kernel<T><<<(unsigned)((nrows + 1) / 2), thr, sm, s>>>(phys, dst, nx, nrows, scale, tw_x);
    }
}

template <typename T>
void fft_phys_to_spec(const T* phys, typename CplxOf<T>::type* spec, typename CplxOf<T>::type* tmp,
                      int nx, int ny, int nplanes, const double* tw_x, const double* tw_y, cudaStream_t s,
                      const T* mul) {
    typedef typename CplxOf<T>::type CT;
    const int H = nx / 2 + 1;
    const long long nrows = (long long)ny * nplanes;
    CT* dst = (ny == 1) ? spec : tmp;
    const T scale = (T)(1.0 / ((double)nx * ny));
    rows_forward<T>(phys, dst, nx, nrows, scale, tw_x, s);
    const int Ry = sq_radix(ny);
    if (ny > 1 && Ry) {
        const int NC = 256 / Ry, ntile = (H + NC - 1) / NC;
        const size_t smc = (size_t)ny * NC * sizeof(CT);
        if (Ry == 16) {
            set_smem<T>((const void*)cols_fft_sq_kernel<T, 16>, smc);
            cols_fft_sq_kernel<T, 16><<<(unsigned)(ntile * (long long)nplanes), 256, smc, s>>>(tmp, spec, H, (T)-1,
                                                                                             tw_y, nplanes, 0LL, mul);
        } else {
            set_smem<T>((const void*)cols_fft_sq_kernel<T, 8>, smc);
            cols_fft_sq_kernel<T, 8><<<(unsigned)(ntile * (long long)nplanes), 256, smc, s>>>(tmp, spec, H, (T)-1,
                                                                                            tw_y, nplanes, 0LL, mul);
        }
    } else if (ny > 1) {
        int W = col_tile(ny);
        size_t sm2 = 2 * (size_t)W * ny * sizeof(CT);
        set_smem<T>((const void*)cols_fft_kernel<T>, sm2);
        int ntile = (H + W - 1) / W;
        cols_fft_kernel<T><<<(unsigned)(ntile * (long long)nplanes), 256, sm2, s>>>(tmp, spec, ny, H, W, (T)-1, tw_y,
                                                                                   nplanes, 0LL);
    }
    if (mul && !(ny > 1 && Ry)) {
        const long long n = (long long)nplanes * ny * H;
        spec_mul_kernel<T><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(spec, mul, ny * H, n);
    }
}

// rows of H complex -> rows of nx reals (the inverse row pass of fft_spec_to_phys_g)
template <typename T>
static void rows_inverse(const typename CplxOf<T>::type* src, T* phys, int nx, int ny, long long nrows,
                         int rppg, long long rgs, const double* tw_x, cudaStream_t s) {
    typedef typename CplxOf<T>::type CT;
    const int Rx = sq_radix(nx);
    const long long npairs = (nrows + 1) / 2;
    if (Rx == 16) {
        const size_t sm = (size_t)16 * 16 * 17 * sizeof(CT);
        set_smem<T>((const void*)rows_c2r_sq_kernel<T, 16>, sm);
        rows_c2r_sq_kernel<T, 16><<<(unsigned)((npairs + 15) / 16), 256, sm, s>>>(src, phys, nrows, tw_x, ny, rppg, rgs);
        return;
    }
    if (Rx == 8) {
        const size_t sm = (size_t)32 * 8 * 9 * sizeof(CT);
        set_smem<T>((const void*)rows_c2r_sq_kernel<T, 8>, sm);
        rows_c2r_sq_kernel<T, 8><<<(unsigned)((npairs + 31) / 32), 256, sm, s>>>(src, phys, nrows, tw_x, ny, rppg, rgs);
        return;
    }
    size_t sm = 2 * (size_t)nx * sizeof(CT);
    int thr = nx / 2 < 256 ? (nx / 2 < 32 ? 32 : nx / 2) : 256;
    set_smem<T>((const void*)rows_c2r_kernel<T>, sm);
    rows_c2r_kernel<T><<<(unsigned)npairs, thr, sm, s>>>(src, phys, nx, nrows, tw_x, ny, rppg, rgs);
}

template <typename T>
void fft_spec_to_phys_g(const typename CplxOf<T>::type* spec, int ppg, long long gstride, T* phys,
                        typename CplxOf<T>::type* tmp, int nx, int ny, int nplanes, const double* tw_x,
                        const double* tw_y, cudaStream_t s) {
    typedef typename CplxOf<T>::type CT;
    const int H = nx / 2 + 1;
    const long long nrows = (long long)ny * nplanes;
    const CT* src = spec;
    int rppg = ppg;
    long long rgs = gstride;
    if (ny > 1) {
        const int Ry = sq_radix(ny);
        const unsigned blocks16 = (unsigned)(((H + 15) / 16) * (long long)nplanes);
        const unsigned blocks8 = (unsigned)(((H + 31) / 32) * (long long)nplanes);
        if (Ry == 16) {
            const size_t sm2 = (size_t)16 * 16 * 16 * sizeof(CT);
            set_smem<T>((const void*)cols_fft_sq_kernel<T, 16>, sm2);
            cols_fft_sq_kernel<T, 16><<<blocks16, 256, sm2, s>>>(spec, tmp, H, (T)1, tw_y, ppg, gstride, nullptr);
        } else if (Ry == 8) {
            const size_t sm2 = (size_t)8 * 8 * 32 * sizeof(CT);
            set_smem<T>((const void*)cols_fft_sq_kernel<T, 8>, sm2);
            cols_fft_sq_kernel<T, 8><<<blocks8, 256, sm2, s>>>(spec, tmp, H, (T)1, tw_y, ppg, gstride, nullptr);
        } else {
            int W = col_tile(ny);
            size_t sm2 = 2 * (size_t)W * ny * sizeof(CT);
            set_smem<T>((const void*)cols_fft_kernel<T>, sm2);
            int ntile = (H + W - 1) / W;
            cols_fft_kernel<T><<<(unsigned)(ntile * (long long)nplanes), 256, sm2, s>>>(spec, tmp, ny, H, W, (T)1, tw_y,
                                                                                       ppg, gstride);
        }
        src = tmp;
        rppg = nplanes;      // tmp is contiguous
        rgs = 0;
    }
    rows_inverse<T>(src, phys, nx, ny, nrows, rppg, rgs, tw_x, s);
}

// phys -> out through the half spectrum times the real pencil multiplier
// mul[ky][kx] (damping, horizontal filter).  For ny = 64 or 256 the column
// passes run as one kernel in place on tmp (3 launches); otherwise as
// fft_phys_to_spec + fft_spec_to_phys through spec (4 or 5).  Returns the
// number of launches.
template <typename T>
int fft_filter_phys(const T* phys, T* out, typename CplxOf<T>::type* spec, typename CplxOf<T>::type* tmp, int nx,
                    int ny, int nplanes, const double* tw_x, const double* tw_y, cudaStream_t s, const T* mul) {
    typedef typename CplxOf<T>::type CT;
    const int Ry = sq_radix(ny);
    if (!(ny > 1 && Ry)) {
        fft_phys_to_spec<T>(phys, spec, tmp, nx, ny, nplanes, tw_x, tw_y, s, mul);
        fft_spec_to_phys<T>(spec, out, tmp, nx, ny, nplanes, tw_x, tw_y, s);
        return ny > 1 ? 5 : 3;
    }
    const int H = nx / 2 + 1;
    const long long nrows = (long long)ny * nplanes;
    rows_forward<T>(phys, tmp, nx, nrows, (T)(1.0 / ((double)nx * ny)), tw_x, s);
    const int NC = 256 / Ry, ntile = (H + NC - 1) / NC;
    const size_t smc = (size_t)ny * NC * sizeof(CT);
    if (Ry == 16) {
        set_smem<T>((const void*)cols_filter_sq_kernel<T, 16>, smc);
        cols_filter_sq_kernel<T, 16><<<(unsigned)(ntile * (long long)nplanes), 256, smc, s>>>(tmp, H, tw_y, mul);
    } else {
        set_smem<T>((const void*)cols_filter_sq_kernel<T, 8>, smc);
        cols_filter_sq_kernel<T, 8><<<(unsigned)(ntile * (long long)nplanes), 256, smc, s>>>(tmp, H, tw_y, mul);
    }
    rows_inverse<T>(tmp, out, nx, ny, nrows, nplanes, 0LL, tw_x, s);
    return 3;
}

template <typename T>
void fft_spec_to_phys(const typename CplxOf<T>::type* spec, T* phys, typename CplxOf<T>::type* tmp,
                      int nx, int ny, int nplanes, const double* tw_x, const double* tw_y, cudaStream_t s) {
    fft_spec_to_phys_g<T>(spec, nplanes, 0LL, phys, tmp, nx, ny, nplanes, tw_x, tw_y, s);
}

// out = out + i kx fx + i ky fy   (fy may be null)
template <typename T>
__global__ void spec_combine_kernel(typename CplxOf<T>::type* out, const typename CplxOf<T>::type* fx,
                                    const typename CplxOf<T>::type* fy, const T* __restrict__ pt, int M,
                                    long long n, long long out_ss, long long in_ss) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    out += blockIdx.y * out_ss;
    fx += blockIdx.y * in_ss;
    if (fy) fy += blockIdx.y * in_ss;
    int m = (int)(t % M);
    typename CplxOf<T>::type d = imul(pt[PT_KX * (long long)M + m], fx[t]);
    if (fy) d = d + imul(pt[PT_KY * (long long)M + m], fy[t]);
    out[t] = d + out[t];
}

// out(z) = in(z) * zt[row][z]
template <typename T>
__global__ void spec_scale_z_kernel(typename CplxOf<T>::type* out, const typename CplxOf<T>::type* in,
                                    const T* __restrict__ zt, int row, int M, int nz, long long out_ss,
                                    long long in_ss) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)M * nz) return;
    out += blockIdx.y * out_ss;
    in += blockIdx.y * in_ss;
    int z = (int)(t / M);
    out[t] = in[t] * zt[row * nz + z];
}

// which: 0 -> i kx * in, 1 -> i ky * in, 2 -> damping rate * in, 3 -> horizontal filter * in
template <typename T>
__global__ void spec_dxdy_kernel(typename CplxOf<T>::type* out, const typename CplxOf<T>::type* in,
                                 const T* __restrict__ pt, int which, int M, long long n, long long out_ss,
                                 long long in_ss) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    out += blockIdx.y * out_ss;
    in += blockIdx.y * in_ss;
    int m = (int)(t % M);
    if (which == 0) out[t] = imul(pt[PT_KX * (long long)M + m], in[t]);
    else if (which == 1) out[t] = imul(pt[PT_KY * (long long)M + m], in[t]);
    else if (which == 2) out[t] = pt[PT_DAMP * (long long)M + m] * in[t];
    else out[t] = pt[PT_HF * (long long)M + m] * in[t];
}

// Sensitivity-kernel accumulation, kernels.f90:276-311, for nsrc sources at
// once.  fwd planes (field stride fwd_fs, source stride N): 0 div(f_xi), 1-3
// f_acc (x,y,z), 4-6 f_xi (x,y,z); adj planes (stride adj_fs): 0 div(a_v), 1-3
// a_v, 4-6 grad(g a_vz).  acc [src][3][N]: kernelc2, kernelrho, hessian, FP64.
// The time integral is FP64; the per-snapshot products are formed in T (the
// fields' own precision).
template <typename T>
__global__ void kernel_accum_kernel(double* __restrict__ acc, const T* __restrict__ fwd, long long fwd_fs,
                                    const T* __restrict__ adj, long long adj_fs, const double* __restrict__ zt64,
                                    long long NP, int nz, int use_y, int nsrc, const double* __restrict__ c2f) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long N = NP * nz;
    if (t >= N * nsrc) return;
    const long long g = t / N, i = t - g * N;
    const int z = (int)(i / NP);
    double* A = acc + g * 3 * N;
    const T zero = (T)0;
    const T f1 = fwd[t], fax = fwd[fwd_fs + t], fay = use_y ? fwd[2 * fwd_fs + t] : zero, faz = fwd[3 * fwd_fs + t];
    const T fxx = fwd[4 * fwd_fs + t], fxy = use_y ? fwd[5 * fwd_fs + t] : zero, fxz = fwd[6 * fwd_fs + t];
    const T a1 = adj[t], avx = adj[adj_fs + t], avy = use_y ? adj[2 * adj_fs + t] : zero, avz = adj[3 * adj_fs + t];
    const T d31 = adj[4 * adj_fs + t], d32 = use_y ? adj[5 * adj_fs + t] : zero, d33 = adj[6 * adj_fs + t];
    if constexpr (sizeof(T) == 8) {
        const double c2 = c2f ? c2f[i] : zt64[ZT_C2 * nz + z], gr = zt64[ZT_GRAW * nz + z];
        A[2 * N + i] = A[2 * N + i] + faz * faz + fax * fax + fay * fay;
        const double t1 = f1 * a1;
        A[i] = A[i] + t1;
        double kr = A[N + i] + t1 * c2 + faz * avz + fax * avx + fay * avy;
        kr = kr - gr * fxz * a1 + (fxx * d31 + fxy * d32 + fxz * d33);
        A[N + i] = kr;
    } else {
        const T c2 = (T)(c2f ? c2f[i] : zt64[ZT_C2 * nz + z]), gr = (T)zt64[ZT_GRAW * nz + z];
        const T h = faz * faz + fax * fax + fay * fay;
        const T t1 = f1 * a1;
        const T kr = t1 * c2 + faz * avz + fax * avx + fay * avy - gr * fxz * a1 + (fxx * d31 + fxy * d32 + fxz * d33);
        A[2 * N + i] += (double)h;
        A[i] += (double)t1;
        A[N + i] += (double)kr;
    }
}

// Final scaling kernels.f90:523-539, optionally summed over nsum slots
__global__ void kernel_finish_kernel(double* __restrict__ out, const double* __restrict__ acc,
                                     const double* __restrict__ zt64, long long NP, int nz, double scale_c,
                                     double scale_r, int nsum, long long acc_ss, const double* __restrict__ r0f,
                                     const double* __restrict__ c2f) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long N = NP * nz;
    if (t >= N) return;
    const int z = (int)(t / NP);
    const double r0 = r0f ? r0f[t] : zt64[ZT_RHO0 * nz + z], c2 = c2f ? c2f[t] : zt64[ZT_C2 * nz + z];
    double kc = 0, kr = 0, h = 0;
    for (int s = 0; s < nsum; ++s) {
        const double* A = acc + s * acc_ss;
        kc += -A[t] * r0 * c2 * scale_c;
        kr += -r0 * A[N + t] * scale_r;
        h += A[2 * N + t];
    }
    out[t] = kc;
    out[N + t] = kr;
    out[2 * N + t] = h;
}

template <typename T>
__global__ void copy_convert_kernel(T* dst, const double* src, long long n) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) dst[t] = (T)src[t];
}
template <typename T>
__global__ void copy_back_kernel(double* dst, const T* src, long long n) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) dst[t] = (double)src[t];
}

template <typename T>
__global__ void finite_kernel(const T* p, long long n, int* flag) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long stride = (long long)gridDim.x * blockDim.x;
    for (; t < n; t += stride)
        if (!isfinite(p[t])) { *flag = 1; return; }
}

static unsigned nblk(long long n, int b = 256) { return (unsigned)((n + b - 1) / b); }

template <typename T>
void launch_spec_combine(typename CplxOf<T>::type* out, const typename CplxOf<T>::type* fx,
                         const typename CplxOf<T>::type* fy, const T* pt, int M, int nz, int nsrc, long long out_ss,
                         long long in_ss, cudaStream_t s) {
    long long n = (long long)M * nz;
    spec_combine_kernel<T><<<dim3(nblk(n), nsrc), 256, 0, s>>>(out, fx, fy, pt, M, n, out_ss, in_ss);
}
template <typename T>
void launch_spec_scale_z(typename CplxOf<T>::type* out, const typename CplxOf<T>::type* in, const T* zt, int row,
                         int M, int nz, int nsrc, long long out_ss, long long in_ss, cudaStream_t s) {
    spec_scale_z_kernel<T><<<dim3(nblk((long long)M * nz), nsrc), 256, 0, s>>>(out, in, zt, row, M, nz, out_ss, in_ss);
}
template <typename T>
void launch_spec_dxdy(typename CplxOf<T>::type* out, const typename CplxOf<T>::type* in, const T* pt, int which,
                      int M, int nz, int nsrc, long long out_ss, long long in_ss, cudaStream_t s) {
    long long n = (long long)M * nz;
    spec_dxdy_kernel<T><<<dim3(nblk(n), nsrc), 256, 0, s>>>(out, in, pt, which, M, n, out_ss, in_ss);
}
template <typename T>
void launch_kernel_accum(double* acc, const T* fwd, long long fwd_fs, const T* adj, long long adj_fs,
                         const double* zt64, long long NP, int nz, int use_y, int nsrc, cudaStream_t s,
                         const double* c2f) {
    kernel_accum_kernel<T><<<nblk(NP * nz * nsrc), 256, 0, s>>>(acc, fwd, fwd_fs, adj, adj_fs, zt64, NP, nz, use_y,
                                                                nsrc, c2f);
}
void launch_kernel_finish(double* out, const double* acc, const double* zt64, long long NP, int nz, double scale_c,
                          double scale_r, int nsum, long long acc_ss, cudaStream_t s, const double* r0f,
                          const double* c2f) {
    kernel_finish_kernel<<<nblk(NP * nz), 256, 0, s>>>(out, acc, zt64, NP, nz, scale_c, scale_r, nsum, acc_ss, r0f,
                                                       c2f);
}
template <typename T> void launch_copy_convert(T* dst, const double* src, long long n, cudaStream_t s) {
    copy_convert_kernel<T><<<nblk(n), 256, 0, s>>>(dst, src, n);
}
template <typename T> void launch_copy_back(double* dst, const T* src, long long n, cudaStream_t s) {
    copy_back_kernel<T><<<nblk(n), 256, 0, s>>>(dst, src, n);
}
int launch_check_finite_f64(const double* p, long long n, int* flag, cudaStream_t s) {
    finite_kernel<double><<<1024, 256, 0, s>>>(p, n, flag);
    return 0;
}
int launch_check_finite_f32(const float* p, long long n, int* flag, cudaStream_t s) {
    finite_kernel<float><<<1024, 256, 0, s>>>(p, n, flag);
    return 0;
}

#define INST(T)                                                                                                   \
    template int fft_filter_phys<T>(const T*, T*, CplxOf<T>::type*, CplxOf<T>::type*, int, int, int, const double*, \
                                    const double*, cudaStream_t, const T*);                                       \
    template void fft_phys_to_spec<T>(const T*, CplxOf<T>::type*, CplxOf<T>::type*, int, int, int, const double*, \
                                      const double*, cudaStream_t, const T*);                                     \
    template void fft_spec_to_phys<T>(const CplxOf<T>::type*, T*, CplxOf<T>::type*, int, int, int, const double*, \
                                      const double*, cudaStream_t);                                               \
    template void fft_spec_to_phys_g<T>(const CplxOf<T>::type*, int, long long, T*, CplxOf<T>::type*, int, int, \
                                        int, const double*, const double*, cudaStream_t);                         \
    template void launch_spec_combine<T>(CplxOf<T>::type*, const CplxOf<T>::type*, const CplxOf<T>::type*,       \
                                         const T*, int, int, int, long long, long long, cudaStream_t);            \
    template void launch_spec_scale_z<T>(CplxOf<T>::type*, const CplxOf<T>::type*, const T*, int, int, int, int, \
                                         long long, long long, cudaStream_t);                                     \
    template void launch_spec_dxdy<T>(CplxOf<T>::type*, const CplxOf<T>::type*, const T*, int, int, int, int,    \
                                      long long, long long, cudaStream_t);                                        \
    template void launch_kernel_accum<T>(double*, const T*, long long, const T*, long long, const double*,       \
                                         long long, int, int, int, cudaStream_t, const double*);                  \
    template void launch_copy_convert<T>(T*, const double*, long long, cudaStream_t);                             \
    template void launch_copy_back<T>(double*, const T*, long long, cudaStream_t);
INST(double)
INST(float)
