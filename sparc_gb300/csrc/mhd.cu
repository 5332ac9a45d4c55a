// Linearised MHD in the displacement form, option 10 (MP_MHD_PML_3D_DISPL,
// displacement.f90:663-849), on a background that varies in x and y (a
// magnetic flux tube).  The background breaks the per-mode structure of the
// quiet-Sun path, so here the state lives in physical space: each
// [source][field] slot of the context holds one dense (nz, ny, nx) real
// field, and a stage takes its 21 derivatives explicitly:
//   d/dx  two real rows packed as one complex row, shared-memory FFT, times
//         i k normx 2 pi stretchx (the reference's eyekx * stretchx, Nyquist
//         dropped as its c2r does), inverse FFT  (derivatives.f90:28-58);
//   d/dy  two adjacent x-columns packed as one complex column, the same
//         along y (derivatives.f90:62-170); the derivative has a real kernel,
//         so it acts on the packed real and imaginary parts separately;
//   d/dz  DBYD2 on real pencils with the host-factorised MTRIDAG.
// Point-wise kernels form the fluxes, div, p', rho', the induced field b,
// curl b, the Lorentz forces, the sponge and gravity; DAMP_VELOCITY and the
// horizontal filter go through the normalised 2-D transforms and the same
// pencil multipliers as the quiet path.  The PML is bottom-only with six
// auxiliaries (psi_vz, psi_p, psi_dzbx, psi_dzby, psi_induction_bx,
// psi_induction_by; initialize.f90:487-490,560-566); the top has the sponge
// over the last 36 planes.
#include <cmath>
#include <cstring>
#include <vector>
#include <algorithm>

#include "ctx.cuh"

namespace {

// background fields (T, N values each)
enum { MB_BOX, MB_BOY, MB_BOZ, MB_CBOX, MB_CBOY, MB_CBOZ, MB_GP0X, MB_GP0Y, MB_GP0Z, MB_GR0X, MB_GR0Y, MB_GR0Z,
       MB_C2RHO0, MB_RHO0, MB_RHOINV, MB_COUNT };
// stage scratch per source (T, N values each)
enum { MW_T0, MW_T1, MW_T2, MW_T3, MW_T4, MW_T5, MW_F1, MW_F2, MW_F3, MW_DX, MW_DY, MW_DZ, MW_P, MW_R, MW_GPX,
       MW_GPY, MW_GPZ, MW_BX, MW_BY, MW_BZ, MW_DZF1, MW_DZF2, MW_CBX, MW_CBY, MW_CBZ, MW_DZBX, MW_DZBY,
       MW_DMX, MW_DMY, MW_DMZ, MW_COUNT };
// PML auxiliaries of option 10 (scrpml / pmlvars index, initialize.f90:487-490,560-566)
enum { PV_VZ, PV_P, PV_DZBX, PV_DZBY, PV_IBX, PV_IBY, PV_COUNT };

// work fields of a stage of the MHD velocity form (option 8): the eight
// temporaries, the fluxes of v x B0, the eighteen derivatives of the six
// ddxyz calls of pml.f90:106-116 (named for the derivative they hold) and
// the three damping terms
enum { V8_T0, V8_T1, V8_T2, V8_T3, V8_T4, V8_T5, V8_T6, V8_T7, V8_F1, V8_F2, V8_F3,
       V8_DVXDX, V8_DVYDY, V8_DVZDZ, V8_DXF3, V8_GPY, V8_DZF1, V8_GPX, V8_DYF3, V8_DZF2, V8_DXF2, V8_DYBZ,
       V8_DZBX, V8_DXBY, V8_DYBX, V8_GPZ, V8_DXBZ, V8_DYF1, V8_DZBY, V8_DMX, V8_DMY, V8_DMZ, V8_COUNT };

}  // namespace

struct MhdState {
    void* bg = nullptr;        // [MB_COUNT][N] T
    void* pab = nullptr;       // [2][nzpml*NP] T: a_z, b_z of the PML planes (pmlindex order)
    void* g = nullptr;         // [nz] T: gravity with the PML decay of the (1,1) column
    void* sponge = nullptr;    // [nz] T: spongez (PERIODIC: spongexyz(:,:,k) = spongez(k))
    int* plane = nullptr;      // [NP] 0-based source plane of each pixel
    int* plane_obs = nullptr;  // [NP] 0-based observation plane of each pixel (surface records)
    void* dw = nullptr;        // [NP] T: delta_width_2d
    void* rx = nullptr;        // [nx] T: d/dx multipliers of the packed complex FFT
    void* ry = nullptr;        // [ny] T
    void* work = nullptr;      // [S][MW_COUNT][N] T ([S][V8_COUNT][N] in option 8)
    void* pml = nullptr;       // [S][6][nzpml*NP] T (pmlvars)
    void* spml = nullptr;      // [S][6][nzpml*NP] T (scrpml)
    void* spec = nullptr;      // one spectral field (nz*M complex T): damping / filter transforms
    bool have_bg = false;
    // sensitivity kernels of the 2-D form (kernels.f90:99-133, 337-453)
    void* kbox = nullptr;      // [N] T: B_x of kernel mode, -ddzkern(psi, 0) / dimb
    void* kcby = nullptr;      // [N] T: (curl B0)_y of kernel mode (CURL_KERN)
    double* kc2 = nullptr;     // [N] c^2 (non-dimensional) for the kernel products and scaling
    double* krho = nullptr;    // [N] rho0 (non-dimensional)
    double* rx64 = nullptr;    // [nx] FP64 d/dx multipliers (kernel scaling in FP64)
    double* kbacc = nullptr;   // [S][2][N] B-field kernel sums (x, z)
    // a second stream for derivative launches of a stage that are independent
    // of the ones on the context's stream (fork / join through two events)
    cudaStream_t s2 = nullptr;
    cudaEvent_t evf = nullptr, evj = nullptr;
    bool zchunk_scalar = false;   // FP32 z solve with one pencil per lane (SPARC_ZCHUNK_SCALAR, for the tests)
    ~MhdState() {
        if (evf) cudaEventDestroy(evf);
        if (evj) cudaEventDestroy(evj);
        if (s2) cudaStreamDestroy(s2);
    }
};

namespace {

template <typename T>
__device__ __forceinline__ typename CplxOf<T>::type imul_c(T k, typename CplxOf<T>::type z) {
    typename CplxOf<T>::type r;
    r.x = -k * z.y;
    r.y = k * z.x;
    return r;
}

// d/dx of nrows rows of nx reals (rows r = plane*ny + y, dense), two rows per CTA
template <typename T>
__global__ void rowderiv_kernel(const T* __restrict__ in, T* __restrict__ out, int nx, long long nrows,
                                const T* __restrict__ rx, const double* __restrict__ tw) {
    typedef typename CplxOf<T>::type CT;
    extern __shared__ __align__(16) unsigned char smraw[];
    CT* b0 = (CT*)smraw;
    CT* b1 = b0 + nx;
    const long long r0 = 2LL * blockIdx.x, r1 = r0 + 1;
    const bool has1 = r1 < nrows;
    for (int i = threadIdx.x; i < nx; i += blockDim.x) {
        CT v;
        v.x = in[r0 * nx + i];
        v.y = has1 ? in[r1 * nx + i] : (T)0;
        b0[i] = v;
    }
    __syncthreads();
    CT* Z = smem_fft<T, CT>(b0, b1, nx, 1, (T)-1, tw);
    for (int k = threadIdx.x; k < nx; k += blockDim.x) Z[k] = imul_c<T>(rx[k], Z[k]);
    __syncthreads();
    CT* Y = smem_fft<T, CT>(Z, Z == b0 ? b1 : b0, nx, 1, (T)1, tw);
    for (int i = threadIdx.x; i < nx; i += blockDim.x) {
        out[r0 * nx + i] = Y[i].x;
        if (has1) out[r1 * nx + i] = Y[i].y;
    }
}

// ---- spectral derivative of packed lines of length n = R*R (R = 8, 16) ------
// Thread r holds v[n1] = z[R n1 + r] of one packed line z (two real lines as
// real and imaginary parts).  Forward two-pass DFT (n = R n1 + n2, k = k1 +
// R k2: thread n2 does the DFT over n1, twiddle W^(n2 k1), exchange, thread k1
// the DFT over n2), times i*mul[k], then the inverse in the mirrored order
// (thread k1: DFT over k2, twiddle W^-(n2 k1), exchange, thread n2: DFT over
// k1), so that on return v[n1] holds the derivative at R n1 + r again.  The
// derivative operator is real, so the two packed lines stay separate.
// zs(a, b) is the exchange cell (row a, column b) of this line's R x R tile.
template <typename T, typename CT, int R, typename ZS>
__device__ __forceinline__ void deriv_sq(CT (&v)[R], int r, ZS zs, const T* __restrict__ mul,
                                         const double* __restrict__ tw) {
    constexpr int n = R * R;
    CT wf[R / 2], wi[R / 2];
    #pragma unroll
    for (int j = 0; j < R / 2; ++j) {
        wf[j] = tw_n<T, CT>(tw, j * R, n, (T)-1);
        wi[j] = tw_n<T, CT>(tw, j * R, n, (T)1);
    }
    reg_dft<CT, R>(v, wf);
    #pragma unroll
    for (int k1 = 0; k1 < R; ++k1) {
        CT y = v[brev<R>(k1)];
        if (k1 > 0 && r > 0) y = cmul(y, tw_n<T, CT>(tw, r * k1, n, (T)-1));
        zs(k1, r) = y;
    }
    __syncthreads();
    #pragma unroll
    for (int n2 = 0; n2 < R; ++n2) v[n2] = zs(r, n2);
    __syncthreads();                                   // the tile is rewritten below
    reg_dft<CT, R>(v, wf);
    CT u[R];
    #pragma unroll
    for (int k2 = 0; k2 < R; ++k2) {
        const CT X = v[brev<R>(k2)];
        const T m = __ldg(&mul[r + R * k2]);
        u[k2].x = -m * X.y;
        u[k2].y = m * X.x;
    }
    reg_dft<CT, R>(u, wi);
    #pragma unroll
    for (int n2 = 0; n2 < R; ++n2) {
        CT y = u[brev<R>(n2)];
        if (n2 > 0 && r > 0) y = cmul(y, tw_n<T, CT>(tw, r * n2, n, (T)1));
        zs(n2, r) = y;
    }
    __syncthreads();
    #pragma unroll
    for (int k1 = 0; k1 < R; ++k1) u[k1] = zs(r, k1);
    reg_dft<CT, R>(u, wi);
    #pragma unroll
    for (int n1 = 0; n1 < R; ++n1) v[n1] = u[brev<R>(n1)];
}

// d/dx of nrows dense rows of nx = R*R reals: 256/R row pairs per CTA, R
// threads per pair
template <typename T, int R>
__global__ void __launch_bounds__(256) rowderiv_sq_kernel(const T* __restrict__ in, T* __restrict__ out,
                                                          long long nrows, const T* __restrict__ mul,
                                                          const double* __restrict__ tw) {
    typedef typename CplxOf<T>::type CT;
    constexpr int nx = R * R, NPR = 256 / R;
    extern __shared__ __align__(16) unsigned char smraw[];
    const int r = threadIdx.x % R, pp = threadIdx.x / R;
    CT* Zp = (CT*)smraw + pp * R * (R + 1);
    const long long r0 = 2LL * ((long long)blockIdx.x * NPR + pp), r1 = r0 + 1;
    const bool has0 = r0 < nrows, has1 = r1 < nrows;
    CT v[R];
    #pragma unroll
    for (int n1 = 0; n1 < R; ++n1) {
        v[n1].x = has0 ? in[r0 * nx + R * n1 + r] : (T)0;
        v[n1].y = has1 ? in[r1 * nx + R * n1 + r] : (T)0;
    }
    deriv_sq<T, CT, R>(v, r, [&](int a, int b) -> CT& { return Zp[a * (R + 1) + b]; }, mul, tw);
    #pragma unroll
    for (int n1 = 0; n1 < R; ++n1) {
        if (has0) out[r0 * nx + R * n1 + r] = v[n1].x;
        if (has1) out[r1 * nx + R * n1 + r] = v[n1].y;
    }
}

// d/dy of nplanes dense (ny, nx) planes, ny = R*R: 256/R pairs of adjacent
// x-columns per CTA (read and written as one complex value), R threads per pair
template <typename T, int R>
__global__ void __launch_bounds__(256) colderiv_sq_kernel(const T* __restrict__ in, T* __restrict__ out, int nx,
                                                          const T* __restrict__ mul, const double* __restrict__ tw) {
    typedef typename CplxOf<T>::type CT;
    constexpr int ny = R * R, NC = 256 / R;
    extern __shared__ __align__(16) unsigned char smraw[];
    CT* Z = (CT*)smraw;
    const int npair = nx / 2, ntile = (npair + NC - 1) / NC;
    const long long plane = blockIdx.x / ntile;
    const int c = threadIdx.x % NC, r = threadIdx.x / NC;
    const int cp = (blockIdx.x % ntile) * NC + c;
    const bool cv = cp < npair;
    const CT* src = (const CT*)(in + plane * (long long)ny * nx) + cp;
    CT* dst = (CT*)(out + plane * (long long)ny * nx) + cp;
    CT v[R];
    #pragma unroll
    for (int n1 = 0; n1 < R; ++n1) v[n1] = cv ? src[(long long)(R * n1 + r) * npair] : czero<CT>();
    deriv_sq<T, CT, R>(v, r, [&](int a, int b) -> CT& { return Z[(a * R + b) * NC + c]; }, mul, tw);
    if (cv) {
        #pragma unroll
        for (int n1 = 0; n1 < R; ++n1) dst[(long long)(R * n1 + r) * npair] = v[n1];
    }
}

// d/dy of nplanes dense (ny, nx) planes: W complex columns (2W real x) per CTA
template <typename T>
__global__ void colderiv_kernel(const T* __restrict__ in, T* __restrict__ out, int nx, int ny, int W,
                                const T* __restrict__ ry, const double* __restrict__ tw) {
    typedef typename CplxOf<T>::type CT;
    extern __shared__ __align__(16) unsigned char smraw[];
    CT* b0 = (CT*)smraw;
    CT* b1 = b0 + (long long)W * ny;
    const int ntile = (nx / 2) / W;
    const long long plane = blockIdx.x / ntile;
    const int c0 = (blockIdx.x % ntile) * W;
    const long long base = plane * (long long)ny * nx;
    for (int t = threadIdx.x; t < W * ny; t += blockDim.x) {
        const int y = t / W, c = t - y * W;
        const long long o = base + (long long)y * nx + 2 * (c0 + c);
        CT v;
        v.x = in[o];
        v.y = in[o + 1];
        b0[c * ny + y] = v;
    }
    __syncthreads();
    CT* Z = smem_fft<T, CT>(b0, b1, ny, W, (T)-1, tw);
    for (int t = threadIdx.x; t < W * ny; t += blockDim.x) {
        const int k = t % ny;
        Z[t] = imul_c<T>(ry[k], Z[t]);
    }
    __syncthreads();
    CT* Y = smem_fft<T, CT>(Z, Z == b0 ? b1 : b0, ny, W, (T)1, tw);
    for (int t = threadIdx.x; t < W * ny; t += blockDim.x) {
        const int y = t / W, c = t - y * W;
        const long long o = base + (long long)y * nx + 2 * (c0 + c);
        const CT v = Y[c * ny + y];
        out[o] = v.x;
        out[o + 1] = v.y;
    }
}

// d/dz (DBYD2 with stretch, bc 0 or 1) of real pencils: npix pencils per
// field, nfield fields with stride fstride (grid.y)
// bc 2: the caller-set bottom value is 0; bc 3: the caller-set top value is
// topscale * topsrc(plane nz-1) of the same field index
template <typename T>
__global__ void __launch_bounds__(128) zderiv_phys_kernel(const T* __restrict__ zt, Compact<T> cc,
                                                          const T* __restrict__ in, T* __restrict__ out,
                                                          long long npix, int nz, int bc, long long fstride,
                                                          const T* __restrict__ topsrc, T topscale) {
    const long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= npix) return;
    const T* b = in + blockIdx.y * fstride + m;
    T* o = out + blockIdx.y * fstride + m;
    const T top = topsrc ? topscale * topsrc[blockIdx.y * fstride + (long long)(nz - 1) * npix + m] : (T)0;
    compact_forward<T, T>(nz, bc, [&](int j) { return b[(long long)j * npix]; }, (T)0, top,
                          zt + (ZT_TH + 3 * bc) * nz, zt + (ZT_TH + 3 * bc + 1) * nz, cc, o, npix);
    const T* gam = zt + (ZT_TH + 3 * bc + 2) * nz;
    T ud = o[(long long)(nz - 1) * npix];
    o[(long long)(nz - 1) * npix] = ud * zt[ZT_STRETCH * nz + nz - 1];
    for (int j = nz - 2; j >= 0; --j) {
        ud = o[(long long)j * npix] - gam[j + 1] * ud;
        o[(long long)j * npix] = ud * zt[ZT_STRETCH * nz + j];
    }
}

// DBYD2's right-hand side of row j (0-based) for boundary code bc (the rows of
// compact_forward): interior 6th-order stencil, 5th-order rows 1 and nz-2,
// the bc-dependent closures of rows 0 and nz-1 (caller-set bot / top for bc 2 / 3)
template <typename T, typename Ld>
__device__ __forceinline__ T compact_rhs_row(int j, int nz, int bc, Ld B, T bot, T top, const Compact<T>& c) {
    if (j >= 2 && j <= nz - 3) return c.C1 * (B(j + 1) - B(j - 1)) + c.C2 * (B(j + 2) - B(j - 2));
    if (j == 1 || j == 0) {
        const T R1 = c.Cb[0] * B(0) + c.Cb[1] * B(1) + c.Cb[2] * B(2) + c.Cb[3] * B(3) + c.Cb[4] * B(4);
        if (j == 1) return R1;
        if (bc == 0) return (T)0;
        if (bc == 2) return bot;
        const T R0 = c.Cf[0] * B(0) + c.Cf[1] * B(1) + c.Cf[2] * B(2) + c.Cf[3] * B(3);
        return (c.alpha2 * R0 - c.beta1 * R1) * c.cnst;
    }
    const T Rn2 = -(c.Cb[0] * B(nz - 1) + c.Cb[1] * B(nz - 2) + c.Cb[2] * B(nz - 3) + c.Cb[3] * B(nz - 4) +
                    c.Cb[4] * B(nz - 5));
    if (j == nz - 2) return Rn2;
    if (bc == 0) return (T)0;
    if (bc == 3) return top;
    const T Rn1 = -(c.Cf[0] * B(nz - 1) + c.Cf[1] * B(nz - 2) + c.Cf[2] * B(nz - 3) + c.Cf[3] * B(nz - 4));
    return (c.alpha2 * Rn1 - c.beta1 * Rn2) * c.cnst;
}

// bytes of the five coefficient tables of the paired chunk kernel, rounded up
// so the float2 buffers after them are 8-byte aligned
__host__ __device__ inline size_t zchunk2_tables_bytes(int nz) { return (((size_t)5 * nz + 1) * 4 + 15) & ~(size_t)15; }

// d/dz of dense fields (DBYD2 * stretch) by chunks: 32 pencils per CTA (one
// per lane), NCH warps, warp w owning planes [w*cs, w*cs + cs).  Forward
// elimination y_j = (R_j - low_j y_{j-1}) ibd_j is affine in y_{j-1}: each
// warp eliminates its chunk from zero (y'), keeping the product of the
// multipliers -low_j ibd_j, and after one barrier adds the carry-in composed
// from the chunks below.  The back substitution x_j = y_j - gam_{j+1} x_{j+1}
// runs the same way from the top.  Each warp stages its chunk and two halo
// planes either side in its own rows of shared memory (row i = plane s-2+i);
// the input is read once and the result written once.  The coefficient
// tables are copied to shared memory first.
template <typename T, int NCH>
__global__ void __launch_bounds__(32 * NCH) zderiv_chunk_kernel(const T* __restrict__ zt, Compact<T> cc,
                                                                const T* __restrict__ in, T* __restrict__ out,
                                                                long long npix, int nz, int bc, long long fstride,
                                                                const T* __restrict__ topsrc, T topscale) {
    extern __shared__ __align__(16) unsigned char smraw[];
    const int cs = (nz + NCH - 1) / NCH, rows = cs + 4;
    T* tmf = (T*)smraw;                      // [nz] -low_j ibd_j
    T* tib = tmf + nz;                       // [nz] ibd_j
    T* tlo = tib + nz;                       // [nz] low_j
    T* tga = tlo + nz;                       // [nz+1] gam_j (gam_nz = 0)
    T* tst = tga + nz + 1;                   // [nz] stretch_j
    T* Cy = tst + nz;                        // [NCH][32] chunk-end value
    T* Cp = Cy + NCH * 32;                   // [NCH][32] chunk multiplier product
    T* Yall = Cp + NCH * 32;                 // [NCH][rows][32]
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    {
        const T* low = zt + (ZT_TH + 3 * bc) * nz;
        const T* ibd = zt + (ZT_TH + 3 * bc + 1) * nz;
        const T* gam = zt + (ZT_TH + 3 * bc + 2) * nz;
        for (int j = threadIdx.x; j <= nz; j += blockDim.x) {
            if (j < nz) {
                const T l = j > 0 ? low[j] : (T)0, ib = ibd[j];
                tlo[j] = l;
                tib[j] = ib;
                tmf[j] = -l * ib;
                tst[j] = zt[ZT_STRETCH * nz + j];
            }
            tga[j] = (j > 0 && j < nz) ? gam[j] : (T)0;
        }
    }
    T* Y = Yall + (long long)w * rows * 32 + lane;   // Y[i * 32] = plane s - 2 + i
    const long long m = (long long)blockIdx.x * 32 + lane;
    const bool on = m < npix;
    const T* b = in + blockIdx.y * fstride + (on ? m : 0);
    T* o = out + blockIdx.y * fstride + m;
    const int s = w * cs, e = min(nz, s + cs) - 1;   // empty chunk when s > e
    auto B = [&](int j) -> T { return b[(long long)j * npix]; };
    const T top = (topsrc && on) ? topscale * topsrc[blockIdx.y * fstride + (long long)(nz - 1) * npix + m] : (T)0;
    if (s <= e) {
        // asynchronous copies (cp.async): every plane of the chunk in flight at once
        for (int i = 0; i < e - s + 5; ++i) {
            const int j = s - 2 + i;
            if (j >= 0 && j < nz) {
                const unsigned dst = (unsigned)__cvta_generic_to_shared(Y + i * 32);
                const T* src = b + (long long)j * npix;
                if (sizeof(T) == 4)
                    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(dst), "l"(src) : "memory");
                else
                    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(dst), "l"(src) : "memory");
            } else {
                Y[i * 32] = (T)0;
            }
        }
        asm volatile("cp.async.commit_group;\n" ::: "memory");
        asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    }
    __syncthreads();                         // tables
    // the closures of rows 0, 1 and nz-2, nz-1 from the staged planes (before
    // the forward pass overwrites them), global reads only for planes
    // outside this chunk's staged range
    auto Bs = [&](int j) -> T { return (j >= s - 2 && j <= e + 2) ? Y[(j - s + 2) * 32] : B(j); };
    T Rlo0 = (T)0, Rlo1 = (T)0, Rhi2 = (T)0, Rhi1 = (T)0;
    if (s <= e && s <= 1) {
        Rlo0 = compact_rhs_row<T>(0, nz, bc, Bs, (T)0, top, cc);
        Rlo1 = compact_rhs_row<T>(1, nz, bc, Bs, (T)0, top, cc);
    }
    if (s <= e && e >= nz - 2) {
        Rhi2 = compact_rhs_row<T>(nz - 2, nz, bc, Bs, (T)0, top, cc);
        Rhi1 = compact_rhs_row<T>(nz - 1, nz, bc, Bs, (T)0, top, cc);
    }
    // forward, local; row i of plane j is overwritten with y'_j once the
    // register window holds b_j
    T y = (T)0, pr = (T)1;
    if (s <= e) {
        T wm2 = Y[0], wm1 = Y[32], w0 = Y[64], w1 = Y[96], w2 = Y[128];
        for (int j = s, i = 2; j <= e; ++j, ++i) {
            T R;
            if (j >= 2 && j <= nz - 3) R = cc.C1 * (w1 - wm1) + cc.C2 * (w2 - wm2);
            else R = j == 0 ? Rlo0 : (j == 1 ? Rlo1 : (j == nz - 2 ? Rhi2 : Rhi1));
            y = (R - tlo[j] * y) * tib[j];
            pr = pr * tmf[j];
            wm2 = wm1; wm1 = w0; w0 = w1; w1 = w2;
            if (j < e) w2 = Y[(i + 3) * 32];
            Y[i * 32] = y;
        }
    }
    Cy[w * 32 + lane] = y;
    Cp[w * 32 + lane] = pr;
    __syncthreads();
    T cin = (T)0;
    for (int q = 0; q < w; ++q) cin = Cy[q * 32 + lane] + Cp[q * 32 + lane] * cin;
    // forward fix-up, then backward, local
    T x = (T)0;
    pr = (T)1;
    if (s <= e) {
        if (w > 0) {
            T pj = (T)1;
            for (int j = s, i = 2; j <= e; ++j, ++i) {
                pj = pj * tmf[j];
                Y[i * 32] = Y[i * 32] + pj * cin;
            }
        }
        for (int j = e, i = e - s + 2; j >= s; --j, --i) {
            const T g = tga[j + 1];
            x = Y[i * 32] - g * x;
            pr = pr * (-g);
            Y[i * 32] = x;
        }
    }
    __syncthreads();                         // all chunk-end values of the forward pass are read
    Cy[w * 32 + lane] = x;                   // x' at the chunk's first plane
    Cp[w * 32 + lane] = pr;
    __syncthreads();
    T xin = (T)0;
    for (int q = NCH - 1; q > w; --q) xin = Cy[q * 32 + lane] + Cp[q * 32 + lane] * xin;
    if (s <= e && on) {
        T pj = (T)1;
        for (int j = e, i = e - s + 2; j >= s; --j, --i) {
            pj = pj * (-tga[j + 1]);
            o[(long long)j * npix] = (Y[i * 32] + pj * xin) * tst[j];
        }
    }
}

// zderiv_chunk_kernel<float> with two neighbouring pencils per lane (64 per
// CTA, npix even): the planes move as float2, and the compact right-hand
// side, the two recurrences and the scaling are paired FP32 instructions on
// both pencils.  The coefficient tables and the products of the multipliers
// are shared by the pair.  Same elimination, chunking and carry composition
// as the scalar kernel.
template <int NCH>
__global__ void __launch_bounds__(32 * NCH) zderiv_chunk2_kernel(const float* __restrict__ zt, Compact<float> cc,
                                                                 const float* __restrict__ in,
                                                                 float* __restrict__ out, long long npix, int nz,
                                                                 int bc, long long fstride,
                                                                 const float* __restrict__ topsrc, float topscale) {
    extern __shared__ __align__(16) unsigned char smraw[];
    const int cs = (nz + NCH - 1) / NCH, rows = cs + 4;
    float* tmf = (float*)smraw;              // [nz] -low_j ibd_j
    float* tib = tmf + nz;                   // [nz] ibd_j
    float* tlo = tib + nz;                   // [nz] low_j
    float* tga = tlo + nz;                   // [nz+1] gam_j (gam_nz = 0)
    float* tst = tga + nz + 1;               // [nz] stretch_j
    float2* Cy = (float2*)(smraw + zchunk2_tables_bytes(nz));   // [NCH][32] chunk-end values
    float* Cp = (float*)(Cy + NCH * 32);     // [NCH][32] chunk multiplier products
    float2* Yall = (float2*)(Cp + NCH * 32); // [NCH][rows][32]
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    {
        const float* low = zt + (ZT_TH + 3 * bc) * nz;
        const float* ibd = zt + (ZT_TH + 3 * bc + 1) * nz;
        const float* gam = zt + (ZT_TH + 3 * bc + 2) * nz;
        for (int j = threadIdx.x; j <= nz; j += blockDim.x) {
            if (j < nz) {
                const float l = j > 0 ? low[j] : 0.f, ib = ibd[j];
                tlo[j] = l;
                tib[j] = ib;
                tmf[j] = -l * ib;
                tst[j] = zt[ZT_STRETCH * nz + j];
            }
            tga[j] = (j > 0 && j < nz) ? gam[j] : 0.f;
        }
    }
    float2* Y = Yall + (long long)w * rows * 32 + lane;   // Y[i * 32] = plane s - 2 + i
    const long long m = (long long)blockIdx.x * 64 + 2 * lane;
    const bool on = m < npix;                             // npix even: both pencils or neither
    const float* b = in + blockIdx.y * fstride + (on ? m : 0);
    float* o = out + blockIdx.y * fstride + m;
    const int s = w * cs, e = min(nz, s + cs) - 1;
    auto B = [&](int j) -> float2 { return *(const float2*)(b + (long long)j * npix); };
    float2 top = make_float2(0.f, 0.f);
    if (topsrc && on) {
        const float2 tv = *(const float2*)(topsrc + blockIdx.y * fstride + (long long)(nz - 1) * npix + m);
        top = pmul(bc2(topscale), tv);
    }
    if (s <= e) {
        for (int i = 0; i < e - s + 5; ++i) {
            const int j = s - 2 + i;
            if (j >= 0 && j < nz) {
                const unsigned dst = (unsigned)__cvta_generic_to_shared(Y + i * 32);
                const float* src = b + (long long)j * npix;
                asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(dst), "l"(src) : "memory");
            } else {
                Y[i * 32] = make_float2(0.f, 0.f);
            }
        }
        asm volatile("cp.async.commit_group;\n" ::: "memory");
        asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    }
    __syncthreads();
    auto Bs = [&](int j) -> float2 { return (j >= s - 2 && j <= e + 2) ? Y[(j - s + 2) * 32] : B(j); };
    auto rhs_row = [&](int j) -> float2 {
        return make_float2(compact_rhs_row<float>(j, nz, bc, [&](int k) { return Bs(k).x; }, 0.f, top.x, cc),
                           compact_rhs_row<float>(j, nz, bc, [&](int k) { return Bs(k).y; }, 0.f, top.y, cc));
    };
    const float2 Z2 = make_float2(0.f, 0.f);
    float2 Rlo0 = Z2, Rlo1 = Z2, Rhi2 = Z2, Rhi1 = Z2;
    if (s <= e && s <= 1) { Rlo0 = rhs_row(0); Rlo1 = rhs_row(1); }
    if (s <= e && e >= nz - 2) { Rhi2 = rhs_row(nz - 2); Rhi1 = rhs_row(nz - 1); }
    const float2 C1p = bc2(cc.C1), C2p = bc2(cc.C2);
    float2 y = Z2;
    float pr = 1.f;
    if (s <= e) {
        float2 wm2 = Y[0], wm1 = Y[32], w0 = Y[64], w1 = Y[96], w2 = Y[128];
        for (int j = s, i = 2; j <= e; ++j, ++i) {
            float2 R;
            if (j >= 2 && j <= nz - 3) R = pfma(C2p, psub(w2, wm2), pmul(C1p, psub(w1, wm1)));
            else R = j == 0 ? Rlo0 : (j == 1 ? Rlo1 : (j == nz - 2 ? Rhi2 : Rhi1));
            y = pmul(bc2(tib[j]), pfma(bc2(-tlo[j]), y, R));
            pr = pr * tmf[j];
            wm2 = wm1; wm1 = w0; w0 = w1; w1 = w2;
            if (j < e) w2 = Y[(i + 3) * 32];
            Y[i * 32] = y;
        }
    }
    Cy[w * 32 + lane] = y;
    Cp[w * 32 + lane] = pr;
    __syncthreads();
    float2 cin = Z2;
    for (int q = 0; q < w; ++q) cin = pfma(bc2(Cp[q * 32 + lane]), cin, Cy[q * 32 + lane]);
    float2 x = Z2;
    pr = 1.f;
    if (s <= e) {
        if (w > 0) {
            float pj = 1.f;
            for (int j = s, i = 2; j <= e; ++j, ++i) {
                pj = pj * tmf[j];
                Y[i * 32] = pfma(bc2(pj), cin, Y[i * 32]);
            }
        }
        for (int j = e, i = e - s + 2; j >= s; --j, --i) {
            const float g = tga[j + 1];
            x = pfma(bc2(-g), x, Y[i * 32]);
            pr = pr * (-g);
            Y[i * 32] = x;
        }
    }
    __syncthreads();
    Cy[w * 32 + lane] = x;
    Cp[w * 32 + lane] = pr;
    __syncthreads();
    float2 xin = Z2;
    for (int q = NCH - 1; q > w; --q) xin = pfma(bc2(Cp[q * 32 + lane]), xin, Cy[q * 32 + lane]);
    if (s <= e && on) {
        float pj = 1.f;
        for (int j = e, i = e - s + 2; j >= s; --j, --i) {
            pj = pj * (-tga[j + 1]);
            *(float2*)(o + (long long)j * npix) = pmul(bc2(tst[j]), pfma(bc2(pj), xin, Y[i * 32]));
        }
    }
}

// FILTER_VAR_Z (kernels.f90:845-881) of nfield dense fields in place, one
// thread per pencil: rows 2..nz-1 written (the same stencil as FILTER_VARS_3D)
template <typename T>
__global__ void zfilter_phys_kernel(T* __restrict__ f, long long npix, int nz, long long fstride) {
    const long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= npix) return;
    T* p = f + blockIdx.y * fstride + m;
    zfilter_stream<T, T>(
        nz, 0, [&](int j) { return p[(long long)j * npix]; }, [&](int j, T v) { p[(long long)j * npix] = v; });
}

// a += b
template <typename T>
__global__ void add_kernel(T* __restrict__ a, const T* __restrict__ b, long long n) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) a[t] = a[t] + b[t];
}

// out = in * prof[plane]
template <typename T>
__global__ void zscale_kernel(T* __restrict__ out, const T* __restrict__ in, const T* __restrict__ prof,
                              long long npix, long long n) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) out[t] = in[t] * prof[t / npix];
}

// ---- set-up kernels (FP64) -------------------------------------------------

// READ_IN_FIELD (all_modules.f90:491-505) and the reduction of the field
// (physics.f90:116-129); taper[k] is the REAL*4 factor ((k-nz)/10.)**4 of the
// top eleven planes (1 elsewhere), cq the quiet sound speed
__global__ void mhd_read_kernel(double* rho0, double* c2, double* p0, double* bx, double* by, double* bz,
                                const double* cq, const double* taper, long long NP, int nz, double dimrho,
                                double dimc, double dimb) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= NP * nz) return;
    const int k = (int)(t / NP);
    const double r = rho0[t] / dimrho;
    const double cs = c2[t] / dimc;
    rho0[t] = r;
    c2[t] = pow(cs, 2.0);
    p0[t] = p0[t] / (dimrho * pow(dimc, 2.0));
    double x = bx[t] / dimb, y = by[t] / dimb, z = bz[t] / dimb;
    double red = (pow(z, 2.0) + pow(x, 2.0) + pow(y, 2.0)) / (r * pow(cq[k], 2.0));
    red = 8.0 / (8.0 + red);
    red = red * taper[k];
    const double s = pow(red, 0.5);
    bx[t] = x * s; by[t] = y * s; bz[t] = z * s;
}

// a = -a / d (element-wise)
__global__ void neg_div_kernel(double* a, double d, long long n) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) a[t] = -a[t] / d;
}

// a = s1 * b + s2 * c (element-wise)
__global__ void axpby_kernel(double* a, const double* b, double s1, const double* c, double s2, long long n) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) a[t] = s1 * b[t] + (c ? s2 * c[t] : 0.0);
}

// PML decay of gradp0_z / gradrho0_z and the bottom a_z, b_z (physics.f90:255-297)
__global__ void mhd_pml_kernel(double* gp0z, double* gr0z, double* az, double* bzp, const double* c2,
                               const double* rho0, const double* bx, const double* by, const double* bz,
                               const double* z, const double* alph, long long NP, int nz, int nb, int nt) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= NP * nz) return;
    const int k = (int)(t / NP);        // 0-based plane
    const long long q = t - (long long)k * NP;
    const bool bot = k < nb, top = k >= nz - nt;
    if (!bot && !top) return;
    auto tempin = [&](int kk) {
        const long long i = q + NP * kk;
        return pow(c2[i] + (pow(bx[i], 2.0) + pow(by[i], 2.0) + pow(bz[i], 2.0)) / rho0[i], 0.5);
    };
    double dampz, fdec;
    if (bot) {
        const double r = (z[nb - 1] - z[k]) / (z[nb - 1] - z[0]);
        dampz = 2.0 * 3.0 * 3.0 * tempin(0) / (z[nb - 1] - z[0]) * (r * r);
        fdec = alph[k] / (dampz + alph[k]);
        gp0z[t] *= fdec; gr0z[t] *= fdec;
        az[t] = -dampz;
        bzp[t] = -alph[k] - dampz;
    }
    if (top) {
        const double r = (z[nz - nt] - z[k]) / (z[nz - 1] - z[nz - nt]);
        dampz = 3.0 * 3.0 * tempin(nz - 1) / (z[nz - 1] - z[nz - nt]) * (r * r);
        fdec = alph[k] / (dampz + alph[k]);
        gp0z[t] *= fdec; gr0z[t] *= fdec;
        // pmlindex order: the top planes follow the nb bottom ones (read by
        // option 8; option 10 accounts for the bottom only)
        const long long ip = nb + (k - (nz - nt));
        az[ip * NP + q] = -dampz;
        bzp[ip * NP + q] = -alph[k] - dampz;
    }
}

__global__ void rhoinv_kernel(double* rhoinv, double* c2rho0, const double* rho0, const double* c2, long long n) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    rhoinv[t] = 1.0 / rho0[t];
    c2rho0[t] = c2[t] * rho0[t];
}

template <typename T>
__global__ void to_t_kernel(T* dst, const double* src, long long n) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) dst[t] = (T)src[t];
}

// ---- stage kernels (T) -------------------------------------------------------

struct MhdArgs {
    long long N, NP, FS;   // points per field, per plane; field stride of the state slots
    int nz, nb, nt, nzpml;
    int S;
    int both;              // PML at both ends (options 8, 18) or at the bottom only (option 10)
    int nf;                // fields per state slot (8 in option 8, else 6)
};

// pmlindex of 0-based plane k (PML_BOUNDARY_ACCOUNTING order), -1 outside
__device__ __forceinline__ int pml_plane(const MhdArgs& A, int k) {
    if (k < A.nb) return k;
    if (A.both && k >= A.nz - A.nt) return A.nb + (k - (A.nz - A.nt));
    return -1;
}

// temp = a + beta*scr (step.f90:52-71) into T0..T5, and the fluxes of xi x B0
// (displacement.f90:672-674)
template <typename T>
__global__ void mhd_temp_kernel(const MhdArgs A, const T* __restrict__ a, const T* __restrict__ scr, T beta, int hs,
                                const T* __restrict__ bg, T* __restrict__ work) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= A.N) return;
    const int s = blockIdx.y;
    const T* as = a + (long long)s * 6 * A.FS;
    const T* ss = scr + (long long)s * 6 * A.FS;
    T* w = work + (long long)s * MW_COUNT * A.N;
    T v[6];
    #pragma unroll
    for (int f = 0; f < 6; ++f) {
        v[f] = as[f * A.FS + t];
        if (hs) v[f] = v[f] + beta * ss[f * A.FS + t];
        w[(MW_T0 + f) * A.N + t] = v[f];
    }
    const T box = bg[MB_BOX * A.N + t], boy = bg[MB_BOY * A.N + t], boz = bg[MB_BOZ * A.N + t];
    w[MW_F1 * A.N + t] = -(v[2] * boy - v[1] * boz);
    w[MW_F2 * A.N + t] = -(v[0] * boz - v[2] * box);
    w[MW_F3 * A.N + t] = -(v[1] * box - v[0] * boy);
}

// PML accounting (pml.f90:213-231 form; the bottom planes only in option 10,
// both ends in option 18): rhs = a_z deriv + b_z psi, deriv += psi, with
// psi = pmlvars + beta*scrpml
template <typename T>
__device__ __forceinline__ T pml_bottom(const MhdArgs& A, long long t, int s, int aux, T deriv, const T* __restrict__ pab,
                                        const T* __restrict__ pml, T* __restrict__ spml, T beta, int hs) {
    const int k = (int)(t / A.NP);
    const int ip = pml_plane(A, k);
    if (ip < 0) return deriv;
    const long long q = t - (long long)k * A.NP;
    const long long np = (long long)A.nzpml * A.NP, ipq = (long long)ip * A.NP + q;
    const long long o = ((long long)s * PV_COUNT + aux) * np + ipq;
    T psi = pml[o];
    if (hs) psi = psi + beta * spml[o];
    spml[o] = pab[ipq] * deriv + pab[np + ipq] * psi;
    return deriv + psi;
}

// div, p', rho' (displacement.f90:694-697) after the psi_vz accounting
template <typename T>
__global__ void mhd_div_kernel(const MhdArgs A, const T* __restrict__ bg, T* __restrict__ work, const T* __restrict__ pab,
                               const T* __restrict__ pml, T* __restrict__ spml, T beta, int hs) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= A.N) return;
    const int s = blockIdx.y;
    T* w = work + (long long)s * MW_COUNT * A.N;
    const T dz = pml_bottom<T>(A, t, s, PV_VZ, w[MW_DZ * A.N + t], pab, pml, spml, beta, hs);
    const T div = w[MW_DX * A.N + t] + w[MW_DY * A.N + t] + dz;
    const T xx = w[MW_T0 * A.N + t], xy = w[MW_T1 * A.N + t], xz = w[MW_T2 * A.N + t];
    w[MW_P * A.N + t] = -bg[MB_C2RHO0 * A.N + t] * div - xz * bg[MB_GP0Z * A.N + t] - xx * bg[MB_GP0X * A.N + t] -
                        xy * bg[MB_GP0Y * A.N + t];
    w[MW_R * A.N + t] = -bg[MB_RHO0 * A.N + t] * div - xz * bg[MB_GR0Z * A.N + t] - xx * bg[MB_GR0X * A.N + t] -
                        xy * bg[MB_GR0Y * A.N + t];
}

// psi_p on gradp_z (displacement.f90:704-716), bottom planes only
template <typename T>
__global__ void mhd_pmlp_kernel(const MhdArgs A, T* __restrict__ work, const T* __restrict__ pab,
                                const T* __restrict__ pml, T* __restrict__ spml, T beta, int hs) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= A.N) return;
    const int s = blockIdx.y;
    T* w = work + (long long)s * MW_COUNT * A.N;
    w[MW_GPZ * A.N + t] = pml_bottom<T>(A, t, s, PV_P, w[MW_GPZ * A.N + t], pab, pml, spml, beta, hs);
}

// induced field b (displacement.f90:729-757): psi_induction_bx/by, then
// bx = bx - dzflux2, by = -by + dzflux1, bz = bz - flux3
template <typename T>
__global__ void mhd_b_kernel(const MhdArgs A, T* __restrict__ work, const T* __restrict__ pab, const T* __restrict__ pml,
                             T* __restrict__ spml, T beta, int hs) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= A.N) return;
    const int s = blockIdx.y;
    T* w = work + (long long)s * MW_COUNT * A.N;
    const T dzf2 = pml_bottom<T>(A, t, s, PV_IBX, w[MW_DZF2 * A.N + t], pab, pml, spml, beta, hs);
    const T dzf1 = pml_bottom<T>(A, t, s, PV_IBY, w[MW_DZF1 * A.N + t], pab, pml, spml, beta, hs);
    w[MW_BX * A.N + t] = w[MW_BX * A.N + t] - dzf2;
    w[MW_BY * A.N + t] = -w[MW_BY * A.N + t] + dzf1;
    w[MW_BZ * A.N + t] = w[MW_BZ * A.N + t] - w[MW_F3 * A.N + t];
}

// curl b, the Lorentz forces, sponge, gravity and RHS xi = v
// (displacement.f90:765-813) into scr
// the rest of a stage of MP_MHD_PML_3D_DISPL, point-wise (displacement.f90:
// 759-848): psi_p on d p'/dz and psi_dzbx, psi_dzby (bottom PML), curl b,
// the two Lorentz terms (CROSS, derivatives.f90:471-480), the sponge on the
// top 36 planes, gravity, RHSxi = v, DAMP_VELOCITY (its terms DMX..DMZ were
// transformed after the temporaries), the kernel-mode source on each pixel's
// source plane while the slot's clock is within the forcing gate, and the
// zero top and bottom rows
template <typename T>
__global__ void mhd_rhs_kernel(const MhdArgs A, const T* __restrict__ bg, T* __restrict__ work, const T* __restrict__ pab,
                               const T* __restrict__ pml, T* __restrict__ spml, T beta, int hs, const T* __restrict__ gz,
                               const T* __restrict__ sponge, T* __restrict__ scr, int damp, SlotClock clk,
                               int src_mode, const T* __restrict__ planes, long long plane_ss, int L,
                               const double* __restrict__ series, int nseries, const int* __restrict__ plane,
                               const T* __restrict__ dw) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= A.N) return;
    const int s = blockIdx.y;
    const int k = (int)(t / A.NP);
    const long long q = t - (long long)k * A.NP;
    T* w = work + (long long)s * MW_COUNT * A.N;
    const T gpz = pml_bottom<T>(A, t, s, PV_P, w[MW_GPZ * A.N + t], pab, pml, spml, beta, hs);
    const T dzbx = pml_bottom<T>(A, t, s, PV_DZBX, w[MW_DZBX * A.N + t], pab, pml, spml, beta, hs);
    const T dzby = pml_bottom<T>(A, t, s, PV_DZBY, w[MW_DZBY * A.N + t], pab, pml, spml, beta, hs);
    const T cbx = w[MW_CBX * A.N + t] - dzby;
    const T cby = -w[MW_CBY * A.N + t] + dzbx;
    const T cbz = w[MW_CBZ * A.N + t] - w[MW_F1 * A.N + t];
    const T box = bg[MB_BOX * A.N + t], boy = bg[MB_BOY * A.N + t], boz = bg[MB_BOZ * A.N + t];
    const T ri = bg[MB_RHOINV * A.N + t];
    // CROSS (derivatives.f90:471-480): c = a x b
    T f1 = cby * boz - cbz * boy;
    T f2 = box * cbz - cbx * boz;
    T f3 = cbx * boy - cby * box;
    T rvx = ri * (-w[MW_GPX * A.N + t] + f1);
    T rvy = ri * (-w[MW_GPY * A.N + t] + f2);
    T rvz = ri * (-gpz + f3);
    const T cbox = bg[MB_CBOX * A.N + t], cboy = bg[MB_CBOY * A.N + t], cboz = bg[MB_CBOZ * A.N + t];
    const T bx = w[MW_BX * A.N + t], by = w[MW_BY * A.N + t], bz = w[MW_BZ * A.N + t];
    f1 = cboy * bz - cboz * by;
    f2 = bx * cboz - cbox * bz;
    f3 = cbox * by - cboy * bx;
    rvx = rvx + ri * f1;
    rvy = rvy + ri * f2;
    rvz = rvz + ri * f3;
    T vx = w[MW_T3 * A.N + t], vy = w[MW_T4 * A.N + t], vz = w[MW_T5 * A.N + t];
    if (k >= A.nz - 36) {
        const T sp = sponge[k];
        rvx = rvx - sp * vx;
        rvy = rvy - sp * vy;
        rvz = rvz - sp * vz;
    }
    rvz = rvz - ri * w[MW_R * A.N + t] * gz[k];
    if (damp) {
        rvx = rvx - w[MW_DMX * A.N + t];
        rvy = rvy - w[MW_DMY * A.N + t];
        rvz = rvz - w[MW_DMZ * A.N + t];
    }
    if (src_mode != 0 && k == plane[q]) {
        const int tl = *clk.time - clk.t0[s];
        if (tl >= 0 && tl <= clk.gate) {
            const T* pl = planes + (long long)s * plane_ss + q;
            T F = (T)0;
            if (src_mode == 1) {
                const T wt = (tl < nseries) ? (T)series[(long long)s * nseries + tl] : (T)0;
                F = wt * pl[0];
            } else {
                for (int l = 0; l < 7; ++l) {
                    int id;
                    const double wl = lagrange_weight(clk, tl, L, l, &id);
                    if (id >= 0) F = F + (T)wl * pl[(long long)id * A.NP];
                }
            }
            rvz = rvz + F / bg[MB_RHO0 * A.N + t] * dw[q];
        }
    }
    if (k == 0 || k == A.nz - 1) {
        vx = vy = vz = rvx = rvy = rvz = (T)0;
    }
    T* ss = scr + (long long)s * 6 * A.FS;
    ss[0 * A.FS + t] = vx;
    ss[1 * A.FS + t] = vy;
    ss[2 * A.FS + t] = vz;
    ss[3 * A.FS + t] = rvx;
    ss[4 * A.FS + t] = rvy;
    ss[5 * A.FS + t] = rvz;
}

// a += dt*scr and FILTER_VARS_3D's z filter (physics.f90:755-783) on every
// (source, field, pixel) column
template <typename T>
__global__ void __launch_bounds__(128) mhd_update_kernel(const MhdArgs A, T* __restrict__ a, const T* __restrict__ scr,
                                                         T dt, int mode) {
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= A.NP) return;
    const int s = blockIdx.y / A.nf, f = blockIdx.y % A.nf;
    T* af = a + ((long long)s * A.nf + f) * A.FS + q;
    const T* sf = scr + ((long long)s * A.nf + f) * A.FS + q;
    zfilter_stream<T, T>(
        A.nz, mode, [&](int j) { const long long o = (long long)j * A.NP; return af[o] + dt * sf[o]; },
        [&](int j, T v) { af[(long long)j * A.NP] = v; });
}

template <typename T>
__global__ void mhd_pml_update_kernel(T* pml, const T* spml, T dt, long long n) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) pml[t] = pml[t] + dt * spml[t];
}

// v_z (field fz of nf per slot) of each slot on its observation plane into
// the record buffer (dense planes) when the slot's clock is on the output cadence
template <typename T>
__global__ void mhd_record_kernel(const T* __restrict__ a, T* __restrict__ rec, const int* __restrict__ t0,
                                  const int* __restrict__ time, int steps, int rec_max, long long FS, long long NP,
                                  long long rec_ss, const int* __restrict__ plane, int nf, int fz) {
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int s = blockIdx.y;
    if (q >= NP) return;
    const int tl = *time - t0[s];
    if (tl < 0 || tl % steps != 0) return;
    const int r = tl / steps;
    if (r >= rec_max) return;
    rec[(long long)s * rec_ss + (long long)r * NP + q] = a[((long long)s * nf + fz) * FS + (long long)plane[q] * NP + q];
}

unsigned nb256(long long n) { return (unsigned)((n + 255) / 256); }


template <typename T>
int ddx_launch(sparc_ctx* c, const T* in, T* out, long long nplanes) {
    const int nx = c->P.nx;
    const long long nrows = nplanes * c->P.ny;
    typedef typename CplxOf<T>::type CT;
    if (nx == 256 || nx == 64) {
        const long long rows_per_cta = 2LL * (256 / (nx == 256 ? 16 : 8));
        const unsigned grid = (unsigned)((nrows + rows_per_cta - 1) / rows_per_cta);
        if (nx == 256) {
            const size_t sm = (size_t)16 * 16 * 17 * sizeof(CT);
            cudaFuncSetAttribute((const void*)rowderiv_sq_kernel<T, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
            rowderiv_sq_kernel<T, 16><<<grid, 256, sm, c->stream>>>(in, out, nrows, (const T*)c->mhd->rx, c->tw_x);
        } else {
            const size_t sm = (size_t)32 * 8 * 9 * sizeof(CT);
            rowderiv_sq_kernel<T, 8><<<grid, 256, sm, c->stream>>>(in, out, nrows, (const T*)c->mhd->rx, c->tw_x);
        }
        c->launches++;
        CKL();
        return SPARC_OK;
    }
    const size_t sm = 2 * (size_t)nx * sizeof(typename CplxOf<T>::type);
    const int thr = nx / 2 < 32 ? 32 : (nx / 2 > 256 ? 256 : nx / 2);
    rowderiv_kernel<T><<<(unsigned)((nrows + 1) / 2), thr, sm, c->stream>>>(in, out, nx, nrows, (const T*)c->mhd->rx,
                                                                           c->tw_x);
    c->launches++;
    CKL();
    return SPARC_OK;
}

template <typename T>
int ddy_launch(sparc_ctx* c, const T* in, T* out, long long nplanes) {
    const int nx = c->P.nx, ny = c->P.ny;
    typedef typename CplxOf<T>::type CT;
    if (ny == 256 || ny == 64) {
        const int R = ny == 256 ? 16 : 8, NC = 256 / R;
        const long long ntile = (nx / 2 + NC - 1) / NC;
        const size_t sm = (size_t)R * R * NC * sizeof(CT);
        if (ny == 256) {
            cudaFuncSetAttribute((const void*)colderiv_sq_kernel<T, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
            colderiv_sq_kernel<T, 16><<<(unsigned)(nplanes * ntile), 256, sm, c->stream>>>(in, out, nx, (const T*)c->mhd->ry,
                                                                                        c->tw_y);
        } else {
            cudaFuncSetAttribute((const void*)colderiv_sq_kernel<T, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
            colderiv_sq_kernel<T, 8><<<(unsigned)(nplanes * ntile), 256, sm, c->stream>>>(in, out, nx, (const T*)c->mhd->ry,
                                                                                       c->tw_y);
        }
        c->launches++;
        CKL();
        return SPARC_OK;
    }
    const int W = std::max(1, std::min(nx / 2, 1024 / ny));
    const size_t sm = 2 * (size_t)W * ny * sizeof(typename CplxOf<T>::type);
    colderiv_kernel<T><<<(unsigned)(nplanes * ((nx / 2) / W)), 256, sm, c->stream>>>(in, out, nx, ny, W,
                                                                                   (const T*)c->mhd->ry, c->tw_y);
    c->launches++;
    CKL();
    return SPARC_OK;
}

template <typename T>
Compact<T> cc_of(const sparc_ctx* c) {
    Compact<T> cc;
    cc.C1 = (T)c->cc64.C1; cc.C2 = (T)c->cc64.C2;
    for (int i = 0; i < 5; ++i) cc.Cb[i] = (T)c->cc64.Cb[i];
    for (int i = 0; i < 4; ++i) cc.Cf[i] = (T)c->cc64.Cf[i];
    cc.alpha2 = (T)c->cc64.alpha2; cc.beta1 = (T)c->cc64.beta1; cc.cnst = (T)c->cc64.cnst;
    return cc;
}

// d/dz of nfield fields (stride fstride) with the context's T tables
template <typename T>
int ddz_launch(sparc_ctx* c, const T* zt, const T* in, T* out, int bc, int nfield, long long fstride,
               const T* topsrc = nullptr, T topscale = (T)0) {
    // FP32: chunked solve; FP64: one thread per pencil (the chunked form's
    // extra multiplications cost more on the FP64 pipe than it saves)
    constexpr int NCH = 8;
    const int cs = (c->nz + NCH - 1) / NCH;
    const size_t sm = ((size_t)5 * c->nz + 1 + 2 * NCH * 32 + (size_t)NCH * (cs + 4) * 32) * sizeof(T);
    if constexpr (sizeof(T) == 4) {
        // two pencils per lane when the pencil count is even
        const size_t sm2 = zchunk2_tables_bytes(c->nz) + (size_t)NCH * 32 * (8 + 4) + (size_t)NCH * (cs + 4) * 32 * 8;
        if ((c->NP & 1) == 0 && sm2 <= 200 * 1024 && !(c->mhd && c->mhd->zchunk_scalar)) {
            cudaFuncSetAttribute((const void*)zderiv_chunk2_kernel<NCH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)sm2);
            dim3 g((unsigned)((c->NP + 63) / 64), nfield);
            zderiv_chunk2_kernel<NCH><<<g, 32 * NCH, sm2, c->stream>>>(zt, cc_of<T>(c), in, out, c->NP, c->nz, bc,
                                                                      fstride, topsrc, topscale);
            c->launches++;
            CKL();
            return SPARC_OK;
        }
    }
    if (sizeof(T) == 4 && sm <= 200 * 1024) {
        cudaFuncSetAttribute((const void*)zderiv_chunk_kernel<T, NCH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)sm);
        dim3 g((unsigned)((c->NP + 31) / 32), nfield);
        zderiv_chunk_kernel<T, NCH><<<g, 32 * NCH, sm, c->stream>>>(zt, cc_of<T>(c), in, out, c->NP, c->nz, bc,
                                                                   fstride, topsrc, topscale);
        c->launches++;
        CKL();
        return SPARC_OK;
    }
    dim3 grid((unsigned)((c->NP + 127) / 128), nfield);
    zderiv_phys_kernel<T><<<grid, 128, 0, c->stream>>>(zt, cc_of<T>(c), in, out, c->NP, c->nz, bc, fstride, topsrc,
                                                       topscale);
    c->launches++;
    CKL();
    return SPARC_OK;
}

}  // namespace

int mhd_create(sparc_ctx* c) {
    c->mhd = new MhdState();
    MhdState& m = *c->mhd;
    const size_t es = esz(c);
    int rc;
    m.zchunk_scalar = getenv("SPARC_ZCHUNK_SCALAR") != nullptr;
    CK(cudaStreamCreateWithFlags(&m.s2, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&m.evf, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&m.evj, cudaEventDisableTiming));
    if ((rc = dalloc(c, &m.bg, (size_t)MB_COUNT * c->N * es))) return rc;
    CK(cudaMemsetAsync(m.bg, 0, (size_t)MB_COUNT * c->N * es, c->stream));   // 2-D leaves the y rows at 0
    if ((rc = dalloc(c, &m.pab, (size_t)2 * std::max(c->nzpml, 1) * c->NP * es))) return rc;
    if ((rc = dalloc(c, &m.g, (size_t)c->nz * es))) return rc;
    if ((rc = dalloc(c, &m.sponge, (size_t)c->nz * es))) return rc;
    if ((rc = dalloc(c, (void**)&m.plane, (size_t)c->NP * sizeof(int)))) return rc;
    if ((rc = dalloc(c, (void**)&m.plane_obs, (size_t)c->NP * sizeof(int)))) return rc;
    if ((rc = dalloc(c, &m.dw, (size_t)c->NP * es))) return rc;
    if ((rc = dalloc(c, &m.rx, (size_t)c->P.nx * es))) return rc;
    if ((rc = dalloc(c, &m.ry, (size_t)std::max(c->P.ny, 2) * es))) return rc;
    const int nwork = c->P.option == 8 ? (int)V8_COUNT : (int)MW_COUNT;
    if ((rc = dalloc(c, &m.work, (size_t)c->S * nwork * c->N * es))) return rc;
    const size_t pv = (size_t)c->S * PV_COUNT * std::max(c->nzpml, 1) * c->NP * es;
    if ((rc = dalloc(c, &m.pml, pv))) return rc;
    if ((rc = dalloc(c, &m.spml, pv))) return rc;
    CK(cudaMemsetAsync(m.pml, 0, pv, c->stream));
    CK(cudaMemsetAsync(m.spml, 0, pv, c->stream));   // 2-D never writes psi_dzby, psi_induction_by
    if ((rc = dalloc(c, &m.spec, (size_t)c->fs * csz(c)))) return rc;
    return SPARC_OK;
}

int mhd_set_stream_priority(sparc_ctx* c, int cuda_priority) {
    MhdState& m = *c->mhd;
    CK(cudaStreamSynchronize(m.s2));
    cudaStream_t ns = nullptr;
    CK(cudaStreamCreateWithPriority(&ns, cudaStreamNonBlocking, cuda_priority));
    cudaStreamDestroy(m.s2);
    m.s2 = ns;
    return SPARC_OK;
}

void mhd_destroy(sparc_ctx* c) {
    delete c->mhd;
    c->mhd = nullptr;
}

void* mhd_pml(sparc_ctx* c) { return c->mhd ? c->mhd->pml : nullptr; }
void* mhd_spml(sparc_ctx* c) { return c->mhd ? c->mhd->spml : nullptr; }
const int* mhd_planes(sparc_ctx* c) { return c->mhd ? c->mhd->plane : nullptr; }

// The magnetic parts of mp_Initialize_RHS (physics.f90:62-161, 204-208,
// 255-303, 356-363) in the reference's order; inputs are the 3-D cgs arrays
// READ_IN_FIELD reads, (nz, ny, nx) C order.
int mhd_set_background(sparc_ctx* c, const double* rho, const double* cs, const double* p, const double* bx,
                       const double* by, const double* bz) {
    MhdState& m = *c->mhd;
    const int nz = c->nz, nb = c->P.npmlbot, nt = c->P.npmltop;
    const long long N = c->N, NP = c->NP;
    const std::vector<double>& z = c->zq;
    // FP64 work: 6 inputs, curl (3), horizontal gradients (4), z gradients (2), rhoinv, c2rho0, scratch
    enum { W_RHO, W_C2, W_P, W_BX, W_BY, W_BZ, W_CBX, W_CBY, W_CBZ, W_GP0X, W_GP0Y, W_GR0X, W_GR0Y, W_GP0Z, W_GR0Z,
           W_RI, W_C2R, W_TMP, W_AZ, W_BZP, W_N };
    double* w64 = nullptr;
    int rc = dalloc(c, (void**)&w64, (size_t)W_N * N * 8);
    if (rc) return rc;
    auto W = [&](int i) { return w64 + (size_t)i * N; };
    const double* in[6] = {rho, cs, p, bx, by, bz};
    for (int i = 0; i < 6; ++i)
        if ((rc = upload(c, W(i), in[i], (size_t)N * 8))) return rc;
    // erad_2d / orad_2d (physics.f90:62-87): searched before READ_IN_FIELD,
    // on the density of solar_data (the quiet column) -- the same plane for
    // every pixel; loop bounds clamped to the box
    auto search = [&](int kc) {
        double temp = 1.0;
        int best = kc;
        for (int k = std::max(1, kc - 50); k <= std::min(nz, kc + 10); ++k)
            if (std::fabs(c->rhoq[kc - 1] - c->rhoq[k - 1]) <= temp) {
                temp = std::fabs(c->rhoq[kc - 1] - c->rhoq[k - 1]);
                best = k;
            }
        return best;
    };
    const int erad = search(c->e_rad), orad = search(c->o_rad);
    const int k2 = c->P.compute_adjoint ? orad : erad;
    const int ks = c->P.src_k > 0 ? c->P.src_k : k2;
    std::vector<int> plane(NP, ks - 1), plane_obs(NP, orad - 1);
    const double dw2 = 2.0 / (z[k2] - z[k2 - 2]);
    // spongez (physics.f90:104-108)
    std::vector<double> spz(nz), taper(nz, 1.0), alph(nz), gk(nz);
    for (int k = 0; k < nz; ++k)
        spz[k] = 200.0 / (1.0 + std::exp((R4(1.002) - z[k]) / R4(0.0001))) +
                 300.0 / (1.0 + std::exp((z[k] - (z[0] + R4(0.005))) / R4(0.0005)));
    // ((k-nz)/10.0)**4. in REAL*4 for k = nz-10..nz (physics.f90:123-125)
    for (int k1 = std::max(1, nz - 10); k1 <= nz; ++k1) {
        const float tt = (float)(k1 - nz) / 10.0f;
        taper[k1 - 1] = (double)std::pow(tt, 4.0f);
    }
    // alphaz of the PML planes (physics.f90:269-285)
    for (int k = 1; k <= nz; ++k) {
        double a0 = c->pi * R4(0.005) * c->diml / c->dimc;
        if (k < nb + 1) a0 = c->pi * R4(0.005) * c->diml / c->dimc * (z[k - 1] - z[0]) / (z[nb - 1] - z[0]);
        if (k > nz - nt) a0 = c->pi * R4(0.005) * c->diml / c->dimc * (z[nz - 1] - z[k - 1]) / (z[nz - 1] - z[nz - nt]);
        alph[k - 1] = a0;
    }
    // gravity with the decay of the (1,1) column (physics.f90:287,299), on the host
    {
        const double dimb = std::sqrt(4.0 * c->pi * c->dimc * c->dimc * c->dimrho);
        auto tempin00 = [&](int k) {
            const long long i = (long long)k * NP;
            const double r = rho[i] / c->dimrho, css = cs[i] / c->dimc;
            const double x = bx[i] / dimb, y = by[i] / dimb, zz = bz[i] / dimb;
            double red = (std::pow(zz, 2.0) + std::pow(x, 2.0) + std::pow(y, 2.0)) / (r * std::pow(c->cq[k], 2.0));
            red = 8.0 / (8.0 + red) * taper[k];
            const double sc = std::pow(red, 0.5);
            return std::pow(std::pow(css, 2.0) + (std::pow(x * sc, 2.0) + std::pow(y * sc, 2.0) +
                                                   std::pow(zz * sc, 2.0)) / r, 0.5);
        };
        for (int k = 1; k <= nz; ++k) {
            double fdec = 1.0;
            if (k < nb + 1) {
                const double r = (z[nb - 1] - z[k - 1]) / (z[nb - 1] - z[0]);
                const double dampz = 2.0 * 3.0 * 3.0 * tempin00(0) / (z[nb - 1] - z[0]) * (r * r);
                fdec = alph[k - 1] / (dampz + alph[k - 1]);
            }
            if (k > nz - nt) {
                const double r = (z[nz - nt] - z[k - 1]) / (z[nz - 1] - z[nz - nt]);
                const double dampz = 3.0 * 3.0 * tempin00(nz - 1) / (z[nz - 1] - z[nz - nt]) * (r * r);
                fdec = alph[k - 1] / (dampz + alph[k - 1]);
            }
            gk[k - 1] = c->zt_host[(size_t)ZT_GRAW * nz + k - 1] * fdec;
        }
    }
    double *d_cq = nullptr, *d_taper = nullptr, *d_z = nullptr, *d_alph = nullptr;
    if ((rc = dalloc(c, (void**)&d_cq, nz * 8)) || (rc = dalloc(c, (void**)&d_taper, nz * 8)) ||
        (rc = dalloc(c, (void**)&d_z, nz * 8)) || (rc = dalloc(c, (void**)&d_alph, nz * 8)))
        return rc;
    if ((rc = upload(c, d_cq, c->cq.data(), nz * 8)) || (rc = upload(c, d_taper, taper.data(), nz * 8)) ||
        (rc = upload(c, d_z, z.data(), nz * 8)) || (rc = upload(c, d_alph, alph.data(), nz * 8)))
        return rc;
    const double dimb = std::sqrt(4.0 * c->pi * c->dimc * c->dimc * c->dimrho);
    mhd_read_kernel<<<nb256(N), 256, 0, c->stream>>>(W(W_RHO), W(W_C2), W(W_P), W(W_BX), W(W_BY), W(W_BZ), d_cq,
                                                     d_taper, NP, nz, c->dimrho, c->dimc, dimb);
    CKL();
    // FP64 derivative multipliers for the set-up, then the curl of B0 as the
    // reference forms it (physics.f90:131-159: the d/dz parts are discarded)
    // and the horizontal background gradients (physics.f90:356-363)
    {
        std::vector<double> rx(c->P.nx), ry(std::max(c->P.ny, 2), 0.0);
        for (int k = 0; k < c->P.nx; ++k) {
            const int kk = k < c->P.nx / 2 ? k : (k == c->P.nx / 2 ? 0 : k - c->P.nx);
            rx[k] = (double)kk * c->normx * 2.0 * c->pi * c->stretchx;
        }
        for (int k = 0; k < c->P.ny; ++k) {
            const int kk = k < c->P.ny / 2 ? k : (k == c->P.ny / 2 ? 0 : k - c->P.ny);
            ry[k] = (double)kk * c->normy * 2.0 * c->pi * c->stretchy;
        }
        double *rx64 = nullptr, *ry64 = nullptr;
        if ((rc = dalloc(c, (void**)&rx64, rx.size() * 8)) || (rc = dalloc(c, (void**)&ry64, ry.size() * 8))) return rc;
        if ((rc = upload(c, rx64, rx.data(), rx.size() * 8)) || (rc = upload(c, ry64, ry.data(), ry.size() * 8))) return rc;
        void* rx0 = m.rx; void* ry0 = m.ry;
        m.rx = rx64; m.ry = ry64;                 // FP64 multipliers while setting up
        if ((rc = ddx_launch<double>(c, W(W_BY), W(W_CBZ), nz)) || (rc = ddy_launch<double>(c, W(W_BX), W(W_TMP), nz)))
            return rc;
        axpby_kernel<<<nb256(N), 256, 0, c->stream>>>(W(W_CBZ), W(W_CBZ), 1.0, W(W_TMP), -1.0, N);
        if ((rc = ddy_launch<double>(c, W(W_BZ), W(W_CBX), nz)) || (rc = ddx_launch<double>(c, W(W_BZ), W(W_TMP), nz)))
            return rc;
        axpby_kernel<<<nb256(N), 256, 0, c->stream>>>(W(W_CBY), W(W_TMP), -1.0, nullptr, 0.0, N);
        if ((rc = ddx_launch<double>(c, W(W_RHO), W(W_GR0X), nz)) || (rc = ddy_launch<double>(c, W(W_RHO), W(W_GR0Y), nz)) ||
            (rc = ddx_launch<double>(c, W(W_P), W(W_GP0X), nz)) || (rc = ddy_launch<double>(c, W(W_P), W(W_GP0Y), nz)))
            return rc;
        // d/dz of the background in FP64 (physics.f90:207-208)
        if ((rc = ddz_launch<double>(c, c->zt64, W(W_RHO), W(W_GR0Z), 1, 1, 0)) ||
            (rc = ddz_launch<double>(c, c->zt64, W(W_P), W(W_GP0Z), 1, 1, 0)))
            return rc;
        CKL();
        // multipliers of the element type for the steps
        std::vector<double> rxs = rx, rys = ry;
        m.rx = rx0; m.ry = ry0;
        if (c->f32) {
            std::vector<float> fx(rx.begin(), rx.end()), fy(ry.begin(), ry.end());
            if ((rc = upload(c, m.rx, fx.data(), fx.size() * 4)) || (rc = upload(c, m.ry, fy.data(), fy.size() * 4)))
                return rc;
        } else {
            if ((rc = upload(c, m.rx, rx.data(), rx.size() * 8)) || (rc = upload(c, m.ry, ry.data(), ry.size() * 8)))
                return rc;
        }
    }
    rhoinv_kernel<<<nb256(N), 256, 0, c->stream>>>(W(W_RI), W(W_C2R), W(W_RHO), W(W_C2), N);
    CKL();
    mhd_pml_kernel<<<nb256(N), 256, 0, c->stream>>>(W(W_GP0Z), W(W_GR0Z), W(W_AZ), W(W_BZP), W(W_C2), W(W_RHO),
                                                    W(W_BX), W(W_BY), W(W_BZ), d_z, d_alph, NP, nz, nb, nt);
    CKL();
    // to the element type: background fields, bottom PML coefficients, tables
    const int src_of[MB_COUNT] = {W_BX, W_BY, W_BZ, W_CBX, W_CBY, W_CBZ, W_GP0X, W_GP0Y, W_GP0Z, W_GR0X,
                                  W_GR0Y, W_GR0Z, W_C2R, W_RHO, W_RI};
    // a_z, b_z of all nzpml PML planes in pmlindex order (option 10 reads the bottom nb)
    const long long nbp = (long long)std::max(c->nzpml, 1) * NP, npz = nbp;
    for (int i = 0; i < MB_COUNT; ++i) {
        if (c->f32) to_t_kernel<float><<<nb256(N), 256, 0, c->stream>>>((float*)m.bg + (size_t)i * N, W(src_of[i]), N);
        else to_t_kernel<double><<<nb256(N), 256, 0, c->stream>>>((double*)m.bg + (size_t)i * N, W(src_of[i]), N);
    }
    if (c->f32) {
        to_t_kernel<float><<<nb256(nbp), 256, 0, c->stream>>>((float*)m.pab, W(W_AZ), nbp);
        to_t_kernel<float><<<nb256(nbp), 256, 0, c->stream>>>((float*)m.pab + npz, W(W_BZP), nbp);
    } else {
        to_t_kernel<double><<<nb256(nbp), 256, 0, c->stream>>>((double*)m.pab, W(W_AZ), nbp);
        to_t_kernel<double><<<nb256(nbp), 256, 0, c->stream>>>((double*)m.pab + npz, W(W_BZP), nbp);
    }
    CKL();
    std::vector<double> dwv(NP, dw2);
    if (c->f32) {
        std::vector<float> g32(gk.begin(), gk.end()), s32(spz.begin(), spz.end()), d32(dwv.begin(), dwv.end());
        if ((rc = upload(c, m.g, g32.data(), nz * 4)) || (rc = upload(c, m.sponge, s32.data(), nz * 4)) ||
            (rc = upload(c, m.dw, d32.data(), NP * 4)))
            return rc;
    } else {
        if ((rc = upload(c, m.g, gk.data(), nz * 8)) || (rc = upload(c, m.sponge, spz.data(), nz * 8)) ||
            (rc = upload(c, m.dw, dwv.data(), NP * 8)))
            return rc;
    }
    if ((rc = upload(c, m.plane, plane.data(), NP * sizeof(int)))) return rc;
    if ((rc = upload(c, m.plane_obs, plane_obs.data(), NP * sizeof(int)))) return rc;
    CK(cudaStreamSynchronize(c->stream));
    // release the FP64 set-up buffers
    for (void* pp : {(void*)w64, (void*)d_cq, (void*)d_taper, (void*)d_z, (void*)d_alph}) {
        auto it = std::find(c->allocs.begin(), c->allocs.end(), pp);
        if (it != c->allocs.end()) c->allocs.erase(it);
        cudaFree(pp);
    }
    c->dev_bytes -= (long long)W_N * N * 8 + 4LL * nz * 8;
    m.have_bg = true;
    return SPARC_OK;
}

// ---- option 18 (2-D, ny = 1) ---------------------------------------------------

namespace {

// DBYD1 (dbyd1.f) with ibc = 0 along x for n2 rows of n1: the DBYD2 compact
// scheme with its coefficients in default REAL (the file declares no
// kinds), zero end rows, solved by TRIDAG (tridag.f: Thomas with divisions)
void host_dbyd1_ibc0(std::vector<double>& a, const double* b, int n1, long n2) {
    const float d1i = (float)(n1 - 1);
    const double C1 = (double)(d1i * 7.0f / 9.0f), C2 = (double)(d1i / 36.0f);
    const double B1 = (double)(-43.0f / 96.0f * d1i), B2 = (double)(-5.0f / 6.0f * d1i);
    const double B3 = (double)(9.0f / 8.0f * d1i), B4 = (double)(1.0f / 6.0f * d1i), B5 = (double)(-1.0f / 96.0f * d1i);
    std::vector<double> uppr(n1 + 1, 0.0), lowr(n1 + 1, 0.0), diag(n1 + 1, 1.0), gam(n1 + 1), ud(n1 + 1), r(n1 + 1);
    for (int J = 3; J <= n1 - 2; ++J) uppr[J] = (double)(1.0f / 3.0f);
    uppr[2] = (double)(3.0f / 4.0f);
    uppr[n1 - 1] = (double)(1.0f / 8.0f);
    for (int I = 1; I <= n1; ++I) lowr[I] = uppr[n1 - I + 1];
    lowr[n1] = 0.0;
    a.assign((size_t)n1 * n2, 0.0);
    for (long i = 0; i < n2; ++i) {
        const double* B = b + i * n1 - 1;
        for (int J = 3; J <= n1 - 2; ++J) r[J] = C1 * (B[J + 1] - B[J - 1]) + C2 * (B[J + 2] - B[J - 2]);
        r[2] = B1 * B[1] + B2 * B[2] + B3 * B[3] + B4 * B[4] + B5 * B[5];
        r[n1 - 1] = -(B1 * B[n1] + B2 * B[n1 - 1] + B3 * B[n1 - 2] + B4 * B[n1 - 3] + B5 * B[n1 - 4]);
        r[1] = 0.0;
        r[n1] = 0.0;
        double bet = diag[1];
        ud[1] = r[1] / bet;
        for (int J = 2; J <= n1; ++J) {
            gam[J] = uppr[J - 1] / bet;
            bet = diag[J] - lowr[J] * gam[J];
            ud[J] = (r[J] - lowr[J] * ud[J - 1]) / bet;
        }
        for (int J = n1 - 1; J >= 1; --J) ud[J] = ud[J] - gam[J + 1] * ud[J + 1];
        for (int J = 1; J <= n1; ++J) a[(size_t)i * n1 + J - 1] = ud[J];
    }
}

// physics2d.f90:154-172: non-dimensional background, B = (B_x, B_z) / dimb
__global__ void mhd2d_read_kernel(double* p0, double* rho0, double* c2, double* bx, double* bz, long long n,
                                  double dimrho, double dimc, double dimb) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    bx[t] = bx[t] / dimb;
    bz[t] = bz[t] / dimb;
    p0[t] = p0[t] / (dimrho * pow(dimc, 2.0));
    rho0[t] = rho0[t] / dimrho;
    c2[t] = pow(c2[t] / dimc, 2.0);
}

// PML of physics2d.f90:262-297 with the magnetic wave speed: tempin at
// plane 1 (bottom) and nz-5 (top), factor 3*3 at both ends; a_z, b_z stored
// in pmlindex order; g(k) decayed with the (1,1) column
__global__ void mhd2d_pml_kernel(double* gp0z, double* gr0z, double* az, double* bzp, double* gk, const double* graw,
                                 const double* c2, const double* rho0, const double* bx, const double* bz,
                                 const double* z, const double* alph, long long NP, int nz, int nb, int nt) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= NP * nz) return;
    const int k = (int)(t / NP);
    const long long q = t - (long long)k * NP;
    const bool bot = k < nb, top = k >= nz - nt;
    auto tempin = [&](int kk) {
        const long long i = q + NP * kk;
        return pow(c2[i] + (pow(bx[i], 2.0) + pow(bz[i], 2.0)) / rho0[i], 0.5);
    };
    double fdec = 1.0, dampz = 0.0;
    if (bot) {
        const double r = (z[nb - 1] - z[k]) / (z[nb - 1] - z[0]);
        dampz = 3.0 * 3.0 * tempin(0) / (z[nb - 1] - z[0]) * (r * r);
        fdec = alph[k] / (dampz + alph[k]);
        gp0z[t] *= fdec; gr0z[t] *= fdec;
        az[(long long)k * NP + q] = -dampz;
        bzp[(long long)k * NP + q] = -alph[k] - dampz;
    }
    if (top) {
        const double r = (z[nz - nt] - z[k]) / (z[nz - 1] - z[nz - nt]);
        dampz = 3.0 * 3.0 * tempin(nz - 6) / (z[nz - 1] - z[nz - nt]) * (r * r);
        fdec = alph[k] / (dampz + alph[k]);
        gp0z[t] *= fdec; gr0z[t] *= fdec;
        const long long ip = nb + (k - (nz - nt));
        az[ip * NP + q] = -dampz;
        bzp[ip * NP + q] = -alph[k] - dampz;
    }
    if (q == 0) gk[k] = (bot || top) ? graw[k] * fdec : graw[k];
}

}  // namespace

int mhd2d_set_background(sparc_ctx* c, const double* p, const double* rho, const double* cs, const double* psi) {
    MhdState& m = *c->mhd;
    const int nz = c->nz, nb = c->P.npmlbot, nt = c->P.npmltop, nx = c->P.nx;
    const long long N = c->N, NP = c->NP;
    const std::vector<double>& z = c->zq;
    enum { W_P, W_RHO, W_C2, W_PSI, W_BX, W_BZ, W_CBY, W_TMP, W_RI, W_C2R, W_GR0Z, W_GP0Z, W_GR0X, W_GP0X, W_AZ,
           W_BZP, W_KBX, W_KCY, W_N };
    double* w64 = nullptr;
    int rc = dalloc(c, (void**)&w64, (size_t)W_N * N * 8);
    if (rc) return rc;
    auto W = [&](int i) { return w64 + (size_t)i * N; };
    if ((rc = upload(c, W(W_P), p, N * 8)) || (rc = upload(c, W(W_RHO), rho, N * 8)) ||
        (rc = upload(c, W(W_C2), cs, N * 8)) || (rc = upload(c, W(W_PSI), psi, N * 8)))
        return rc;
    // B_x = -d psi/dz (ddz, bc 1); B_z = DBYD1(psi) * stretchx (physics2d.f90:140-146)
    if ((rc = ddz_launch<double>(c, c->zt64, W(W_PSI), W(W_BX), 1, 1, 0))) return rc;
    axpby_kernel<<<nb256(N), 256, 0, c->stream>>>(W(W_BX), W(W_BX), -1.0, nullptr, 0.0, N);
    std::vector<double> bzh;
    host_dbyd1_ibc0(bzh, psi, nx, (long)nz);
    for (double& v : bzh) v = v * c->stretchx;
    if ((rc = upload(c, W(W_BZ), bzh.data(), N * 8))) return rc;
    const double dimb = std::sqrt(4.0 * c->pi * c->dimc * c->dimc * c->dimrho);
    mhd2d_read_kernel<<<nb256(N), 256, 0, c->stream>>>(W(W_P), W(W_RHO), W(W_C2), W(W_BX), W(W_BZ), N, c->dimrho,
                                                       c->dimc, dimb);
    CKL();
    // curl_y B0 = dBx/dz - dBz/dx (physics2d.f90:180-183), then the gradients
    std::vector<double> rx(nx);
    for (int k = 0; k < nx; ++k) {
        const int kk = k < nx / 2 ? k : (k == nx / 2 ? 0 : k - nx);
        rx[k] = (double)kk * c->normx * 2.0 * c->pi * c->stretchx;
    }
    double* rx64 = nullptr;
    if ((rc = dalloc(c, (void**)&rx64, nx * 8)) || (rc = upload(c, rx64, rx.data(), nx * 8))) return rc;
    void* rx0 = m.rx;
    m.rx = rx64;
    if ((rc = ddz_launch<double>(c, c->zt64, W(W_BX), W(W_CBY), 1, 1, 0)) ||
        (rc = ddx_launch<double>(c, W(W_BZ), W(W_TMP), nz)))
        return rc;
    axpby_kernel<<<nb256(N), 256, 0, c->stream>>>(W(W_CBY), W(W_CBY), 1.0, W(W_TMP), -1.0, N);
    rhoinv_kernel<<<nb256(N), 256, 0, c->stream>>>(W(W_RI), W(W_C2R), W(W_RHO), W(W_C2), N);
    if ((rc = ddz_launch<double>(c, c->zt64, W(W_RHO), W(W_GR0Z), 1, 1, 0)) ||
        (rc = ddz_launch<double>(c, c->zt64, W(W_P), W(W_GP0Z), 1, 1, 0)))
        return rc;
    // PML and gravity
    std::vector<double> alph(nz);
    for (int k = 1; k <= nz; ++k) {
        double a0 = c->pi * R4(0.005) * c->diml / c->dimc;
        if (k < nb + 1) a0 = c->pi * R4(0.005) * c->diml / c->dimc * (z[k - 1] - z[0]) / (z[nb - 1] - z[0]);
        if (k > nz - nt) a0 = c->pi * R4(0.005) * c->diml / c->dimc * (z[nz - 1] - z[k - 1]) / (z[nz - 1] - z[nz - nt]);
        alph[k - 1] = a0;
    }
    double *d_z = nullptr, *d_alph = nullptr, *d_g = nullptr;
    if ((rc = dalloc(c, (void**)&d_z, nz * 8)) || (rc = dalloc(c, (void**)&d_alph, nz * 8)) ||
        (rc = dalloc(c, (void**)&d_g, nz * 8)))
        return rc;
    if ((rc = upload(c, d_z, z.data(), nz * 8)) || (rc = upload(c, d_alph, alph.data(), nz * 8))) return rc;
    mhd2d_pml_kernel<<<nb256(N), 256, 0, c->stream>>>(W(W_GP0Z), W(W_GR0Z), W(W_AZ), W(W_BZP), d_g,
                                                      c->zt64 + (size_t)ZT_GRAW * nz, W(W_C2), W(W_RHO), W(W_BX),
                                                      W(W_BZ), d_z, d_alph, NP, nz, nb, nt);
    CKL();
    // horizontal gradients (physics2d.f90:318-321)
    if ((rc = ddx_launch<double>(c, W(W_RHO), W(W_GR0X), nz)) || (rc = ddx_launch<double>(c, W(W_P), W(W_GP0X), nz)))
        return rc;
    // B0 of kernel mode (kernels.f90:99-133): box = -ddzkern(psi, 0) / dimb
    // (bc 0 and FILTER_VAR_Z, unlike the solve's ddz bc 1), boz as the
    // solve's, curl_y B0 = ddzkern(box, 0) - d boz/dx (CURL_KERN with bcz = 0)
    if ((rc = ddz_launch<double>(c, c->zt64, W(W_PSI), W(W_KBX), 0, 1, 0))) return rc;
    zfilter_phys_kernel<double><<<dim3(nb256(NP), 1), 256, 0, c->stream>>>(W(W_KBX), NP, nz, 0);
    neg_div_kernel<<<nb256(N), 256, 0, c->stream>>>(W(W_KBX), dimb, N);
    if ((rc = ddz_launch<double>(c, c->zt64, W(W_KBX), W(W_KCY), 0, 1, 0))) return rc;
    zfilter_phys_kernel<double><<<dim3(nb256(NP), 1), 256, 0, c->stream>>>(W(W_KCY), NP, nz, 0);
    if ((rc = ddx_launch<double>(c, W(W_BZ), W(W_TMP), nz))) return rc;
    axpby_kernel<<<nb256(N), 256, 0, c->stream>>>(W(W_KCY), W(W_KCY), 1.0, W(W_TMP), -1.0, N);
    CKL();
    if (!m.kc2) {
        if ((rc = dalloc(c, (void**)&m.kc2, N * 8)) || (rc = dalloc(c, (void**)&m.krho, N * 8)) ||
            (rc = dalloc(c, &m.kbox, N * esz(c))) || (rc = dalloc(c, &m.kcby, N * esz(c))))
            return rc;
    }
    CK(cudaMemcpyAsync(m.kc2, W(W_C2), N * 8, cudaMemcpyDeviceToDevice, c->stream));
    CK(cudaMemcpyAsync(m.krho, W(W_RHO), N * 8, cudaMemcpyDeviceToDevice, c->stream));
    if (c->f32) {
        to_t_kernel<float><<<nb256(N), 256, 0, c->stream>>>((float*)m.kbox, W(W_KBX), N);
        to_t_kernel<float><<<nb256(N), 256, 0, c->stream>>>((float*)m.kcby, W(W_KCY), N);
    } else {
        to_t_kernel<double><<<nb256(N), 256, 0, c->stream>>>((double*)m.kbox, W(W_KBX), N);
        to_t_kernel<double><<<nb256(N), 256, 0, c->stream>>>((double*)m.kcby, W(W_KCY), N);
    }
    m.rx64 = rx64;                           // kept for the kernel scaling in FP64
    m.rx = rx0;
    {
        std::vector<double> rxs(rx);
        if (c->f32) {
            std::vector<float> fx(rxs.begin(), rxs.end());
            if ((rc = upload(c, m.rx, fx.data(), nx * 4))) return rc;
        } else if ((rc = upload(c, m.rx, rxs.data(), nx * 8))) {
            return rc;
        }
    }
    // to the element type (the y components and the other curl components stay 0)
    const int dst_of[] = {MB_BOX, MB_BOZ, MB_CBOY, MB_GP0X, MB_GP0Z, MB_GR0X, MB_GR0Z, MB_C2RHO0, MB_RHO0, MB_RHOINV};
    const int src_of[] = {W_BX, W_BZ, W_CBY, W_GP0X, W_GP0Z, W_GR0X, W_GR0Z, W_C2R, W_RHO, W_RI};
    const long long npz = (long long)std::max(c->nzpml, 1) * NP;
    for (int i = 0; i < 10; ++i) {
        if (c->f32) to_t_kernel<float><<<nb256(N), 256, 0, c->stream>>>((float*)m.bg + (size_t)dst_of[i] * N, W(src_of[i]), N);
        else to_t_kernel<double><<<nb256(N), 256, 0, c->stream>>>((double*)m.bg + (size_t)dst_of[i] * N, W(src_of[i]), N);
    }
    if (c->f32) {
        to_t_kernel<float><<<nb256(npz), 256, 0, c->stream>>>((float*)m.pab, W(W_AZ), npz);
        to_t_kernel<float><<<nb256(npz), 256, 0, c->stream>>>((float*)m.pab + npz, W(W_BZP), npz);
        to_t_kernel<float><<<nb256(nz), 256, 0, c->stream>>>((float*)m.g, d_g, nz);
    } else {
        to_t_kernel<double><<<nb256(npz), 256, 0, c->stream>>>((double*)m.pab, W(W_AZ), npz);
        to_t_kernel<double><<<nb256(npz), 256, 0, c->stream>>>((double*)m.pab + npz, W(W_BZP), npz);
        to_t_kernel<double><<<nb256(nz), 256, 0, c->stream>>>((double*)m.g, d_g, nz);
    }
    CKL();
    // source planes: erad_2d = e_rad, orad_2d = o_rad (physics2d.f90:334-341)
    const int k2 = c->P.compute_adjoint ? c->o_rad : c->e_rad;
    const int ks = c->P.src_k > 0 ? c->P.src_k : k2;
    std::vector<int> plane(NP, ks - 1), plane_obs(NP, c->o_rad - 1);
    std::vector<double> dwv(NP, 2.0 / (z[k2] - z[k2 - 2]));
    if (c->f32) {
        std::vector<float> d32(dwv.begin(), dwv.end());
        if ((rc = upload(c, m.dw, d32.data(), NP * 4))) return rc;
    } else if ((rc = upload(c, m.dw, dwv.data(), NP * 8))) {
        return rc;
    }
    if ((rc = upload(c, m.plane, plane.data(), NP * sizeof(int))) ||
        (rc = upload(c, m.plane_obs, plane_obs.data(), NP * sizeof(int))))
        return rc;
    CK(cudaStreamSynchronize(c->stream));
    for (void* pp : {(void*)w64, (void*)d_z, (void*)d_alph, (void*)d_g}) {
        auto it = std::find(c->allocs.begin(), c->allocs.end(), pp);
        if (it != c->allocs.end()) c->allocs.erase(it);
        cudaFree(pp);
    }
    c->dev_bytes -= (long long)W_N * N * 8 + 3LL * nz * 8;
    m.have_bg = true;
    return SPARC_OK;
}

namespace {

// 2-D stage kernels (MP_MHD_PML_2D_DISPL, physics2d.f90:724-943)
template <typename T>
__global__ void mhd2d_div_kernel(const MhdArgs A, const T* __restrict__ bg, T* __restrict__ work, const T* __restrict__ pab,
                                 const T* __restrict__ pml, T* __restrict__ spml, T beta, int hs) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= A.N) return;
    const int s = blockIdx.y;
    T* w = work + (long long)s * MW_COUNT * A.N;
    const T dz = pml_bottom<T>(A, t, s, PV_VZ, w[MW_DZ * A.N + t], pab, pml, spml, beta, hs);
    const T div = w[MW_DX * A.N + t] + dz;
    const T xx = w[MW_T0 * A.N + t], xz = w[MW_T2 * A.N + t];
    w[MW_P * A.N + t] = -bg[MB_C2RHO0 * A.N + t] * div - xz * bg[MB_GP0Z * A.N + t] - xx * bg[MB_GP0X * A.N + t];
    w[MW_R * A.N + t] = -bg[MB_RHO0 * A.N + t] * div - xz * bg[MB_GR0Z * A.N + t] - xx * bg[MB_GR0X * A.N + t];
}

template <typename T>
__global__ void mhd2d_b_kernel(const MhdArgs A, T* __restrict__ work, const T* __restrict__ pab, const T* __restrict__ pml,
                               T* __restrict__ spml, T beta, int hs) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= A.N) return;
    const int s = blockIdx.y;
    T* w = work + (long long)s * MW_COUNT * A.N;
    w[MW_BX * A.N + t] = -pml_bottom<T>(A, t, s, PV_IBX, w[MW_BX * A.N + t], pab, pml, spml, beta, hs);
}

template <typename T>
__global__ void mhd2d_rhs_kernel(const MhdArgs A, const T* __restrict__ bg, T* __restrict__ work, const T* __restrict__ pab,
                                 const T* __restrict__ pml, T* __restrict__ spml, T beta, int hs, const T* __restrict__ gz,
                                 T* __restrict__ scr) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= A.N) return;
    const int s = blockIdx.y;
    const int k = (int)(t / A.NP);
    T* w = work + (long long)s * MW_COUNT * A.N;
    const T dzbx = pml_bottom<T>(A, t, s, PV_DZBX, w[MW_DZBX * A.N + t], pab, pml, spml, beta, hs);
    const T cby = -w[MW_CBY * A.N + t] + dzbx;
    const T box = bg[MB_BOX * A.N + t], boz = bg[MB_BOZ * A.N + t], cboy = bg[MB_CBOY * A.N + t];
    const T ri = bg[MB_RHOINV * A.N + t];
    T rvx = ri * (-w[MW_GPX * A.N + t] + cby * boz);
    T rvz = ri * (-w[MW_GPZ * A.N + t] + (-cby * box));
    rvx = rvx + ri * (cboy * w[MW_BZ * A.N + t]);
    rvz = rvz + ri * (-cboy * w[MW_BX * A.N + t]);
    rvz = rvz - ri * w[MW_R * A.N + t] * gz[k];
    T* ss = scr + (long long)s * 6 * A.FS;
    ss[0 * A.FS + t] = w[MW_T3 * A.N + t];
    ss[1 * A.FS + t] = (T)0;
    ss[2 * A.FS + t] = w[MW_T5 * A.N + t];
    ss[3 * A.FS + t] = rvx;
    ss[4 * A.FS + t] = (T)0;
    ss[5 * A.FS + t] = rvz;
}

// damping of v_x, v_z (DX, DZ), the source while time <= forcing_length *
// cadforcing_step (forward: vr * fwdsource / rho0 * dw; adjoint: forcing * dw
// / rho0), and the zero bottom row (physics2d.f90:897-938)
template <typename T>
__global__ void mhd2d_final_kernel(const MhdArgs A, const T* __restrict__ bg, const T* __restrict__ work, int damp,
                                   T* __restrict__ scr, SlotClock clk, int src_mode, const T* __restrict__ planes,
                                   long long plane_ss, int L, const double* __restrict__ series, int nseries,
                                   const int* __restrict__ plane, const T* __restrict__ dw, int adjoint) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= A.N) return;
    const int s = blockIdx.y;
    const int k = (int)(t / A.NP);
    const long long q = t - (long long)k * A.NP;
    const T* w = work + (long long)s * MW_COUNT * A.N;
    T* ss = scr + (long long)s * 6 * A.FS;
    if (damp) {
        ss[3 * A.FS + t] = ss[3 * A.FS + t] - w[MW_DX * A.N + t];
        ss[5 * A.FS + t] = ss[5 * A.FS + t] - w[MW_DZ * A.N + t];
    }
    if (src_mode != 0 && k == plane[q]) {
        const int tl = *clk.time - clk.t0[s];
        if (tl >= 0 && tl <= clk.gate) {
            const T* pl = planes + (long long)s * plane_ss + q;
            T F = (T)0;
            if (src_mode == 1) {
                const T wt = (tl < nseries) ? (T)series[(long long)s * nseries + tl] : (T)0;
                F = wt * pl[0];
            } else {
                for (int l = 0; l < 7; ++l) {
                    int id;
                    const double wl = lagrange_weight(clk, tl, L, l, &id);
                    if (id >= 0) F = F + (T)wl * pl[(long long)id * A.NP];
                }
            }
            const T r0 = bg[MB_RHO0 * A.N + t];
            ss[5 * A.FS + t] = ss[5 * A.FS + t] + (adjoint ? F * dw[q] / r0 : F / r0 * dw[q]);
        }
    }
    if (k == 0) {
        #pragma unroll
        for (int f = 0; f < 6; ++f) ss[f * A.FS + t] = (T)0;
    }
}

template <typename T>
int mhd2d_stage(sparc_ctx* c, T beta, int hs) {
    MhdState& m = *c->mhd;
    const int S = c->active_n, nz = c->nz;
    MhdArgs A;
    A.N = c->N; A.NP = c->NP; A.FS = 2 * c->fs; A.nz = nz; A.nb = c->P.npmlbot; A.nt = c->P.npmltop;
    A.nzpml = std::max(c->nzpml, 1);
    A.S = S;
    A.both = 1;
    A.nf = 6;
    T* bg = (T*)m.bg;
    T* work = (T*)m.work;
    const T* pab = (const T*)m.pab;
    T* pml = (T*)m.pml;
    T* spml = (T*)m.spml;
    const T* zt = (const T*)c->zt;
    const long long N = c->N, fst = (long long)MW_COUNT * N;
    const dim3 g(nb256(N), S);
    auto Wp = [&](int s, int f) { return work + ((size_t)s * MW_COUNT + f) * N; };
    int rc;
    mhd_temp_kernel<T><<<g, 256, 0, c->stream>>>(A, (const T*)c->a, (const T*)c->scr, beta, hs, bg, work);
    c->launches++;
    CKL();
    // d(xi_x)/dx; d(xi_z)/dz with bc 3, the top value -dxixdx(nz) * unstretch(nz) (physics2d.f90:731-733)
    for (int s = 0; s < S; ++s)
        if ((rc = ddx_launch<T>(c, Wp(s, MW_T0), Wp(s, MW_DX), nz))) return rc;
    const T unstr = (T)c->zt_host[(size_t)ZT_UNSTRETCH * nz + nz - 1];
    if ((rc = ddz_launch<T>(c, zt, Wp(0, MW_T2), Wp(0, MW_DZ), 3, S, fst, Wp(0, MW_DX), -unstr))) return rc;
    mhd2d_div_kernel<T><<<g, 256, 0, c->stream>>>(A, bg, work, pab, pml, spml, beta, hs);
    c->launches++;
    CKL();
    // grad p: ddx(p); ddz(p, bc 2) with the caller-set bottom value 0 (every reachable state)
    for (int s = 0; s < S; ++s)
        if ((rc = ddx_launch<T>(c, Wp(s, MW_P), Wp(s, MW_GPX), nz))) return rc;
    if ((rc = ddz_launch<T>(c, zt, Wp(0, MW_P), Wp(0, MW_GPZ), 2, S, fst))) return rc;
    mhd_pmlp_kernel<T><<<g, 256, 0, c->stream>>>(A, work, pab, pml, spml, beta, hs);
    c->launches++;
    CKL();
    // induction: bx = -(d flux2/dz + psi), bz = d flux2/dx
    for (int s = 0; s < S; ++s)
        if ((rc = ddx_launch<T>(c, Wp(s, MW_F2), Wp(s, MW_BZ), nz))) return rc;
    if ((rc = ddz_launch<T>(c, zt, Wp(0, MW_F2), Wp(0, MW_BX), 0, S, fst))) return rc;
    mhd2d_b_kernel<T><<<g, 256, 0, c->stream>>>(A, work, pab, pml, spml, beta, hs);
    c->launches++;
    CKL();
    // curl_y b = -d bz/dx + (d bx/dz + psi)
    for (int s = 0; s < S; ++s)
        if ((rc = ddx_launch<T>(c, Wp(s, MW_BZ), Wp(s, MW_CBY), nz))) return rc;
    if ((rc = ddz_launch<T>(c, zt, Wp(0, MW_BX), Wp(0, MW_DZBX), 0, S, fst))) return rc;
    mhd2d_rhs_kernel<T><<<g, 256, 0, c->stream>>>(A, bg, work, pab, pml, spml, beta, hs, (const T*)m.g, (T*)c->scr);
    c->launches++;
    CKL();
    const bool damp = c->P.damp_waves != 0;
    if (damp) {
        typedef typename CplxOf<T>::type CT;
        for (int s = 0; s < S; ++s)
            for (int q = 0; q < 2; ++q) {
                const int src = q == 0 ? MW_T3 : MW_T5, dst = q == 0 ? MW_DX : MW_DZ;
                c->launches += fft_filter_phys<T>(Wp(s, src), Wp(s, dst), (CT*)m.spec, (CT*)c->tmp, c->P.nx, 1, nz,
                                                  c->tw_x, c->tw_y, c->stream, (const T*)c->pt + (size_t)PT_DAMP * c->M);
            }
        CKL();
    }
    SlotClock clk;
    memset(&clk, 0, sizeof(clk));
    clk.t0 = c->d_t0; clk.time = c->d_time; clk.freq = c->freq_filtering; clk.two_d = 1;
    clk.gate = c->forcing_length * c->cadforcing_step; clk.num_steps = c->num_steps;
    clk.ts = R4(c->P.timestep); clk.cad = R4(c->P.cadforcing);
    mhd2d_final_kernel<T><<<g, 256, 0, c->stream>>>(A, bg, work, damp ? 1 : 0, (T*)c->scr, clk, c->src_mode,
                                                     (const T*)c->planes, (long long)c->src_L * c->NP, c->src_L,
                                                     c->series, c->nseries, m.plane, (const T*)m.dw,
                                                     c->P.compute_adjoint ? 1 : 0);
    c->launches++;
    CKL();
    return SPARC_OK;
}

}  // namespace

namespace {

// ---- option 8: MP_MHD_PML_3D (pml.f90:80-208), the MHD velocity form -----------
// fields rho, v_x, v_y, v_z, p, b_x, b_y, b_z

// temp = a + beta*scr (step.f90:52-71) into T0..T7 and the fluxes of v x B0
// (pml.f90:93-95)
template <typename T>
__global__ void mhd8_temp_kernel(const MhdArgs A, const T* __restrict__ a, const T* __restrict__ scr, T beta, int hs,
                                 const T* __restrict__ bg, T* __restrict__ work) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= A.N) return;
    const int s = blockIdx.y;
    const T* as = a + (long long)s * 8 * A.FS;
    const T* ss = scr + (long long)s * 8 * A.FS;
    T* w = work + (long long)s * V8_COUNT * A.N;
    T v[8];
    #pragma unroll
    for (int f = 0; f < 8; ++f) {
        v[f] = as[f * A.FS + t];
        if (hs) v[f] = v[f] + beta * ss[f * A.FS + t];
        w[(V8_T0 + f) * A.N + t] = v[f];
    }
    const T box = bg[MB_BOX * A.N + t], boy = bg[MB_BOY * A.N + t], boz = bg[MB_BOZ * A.N + t];
    w[V8_F1 * A.N + t] = -(v[3] * boy - v[2] * boz);
    w[V8_F2 * A.N + t] = -(v[1] * boz - v[3] * box);
    w[V8_F3 * A.N + t] = -(v[2] * box - v[1] * boy);
}

// everything after the derivatives, point-wise: PML_BOUNDARY_ACCOUNTING_3D
// at both ends (pml.f90:213-285), the induction RHS, div, curl b, continuity,
// pressure, the two Lorentz terms (CROSS, derivatives.f90:471-480), gravity,
// the source forcing * source_dep(k) for |k - e_rad| <= 4 (pml.f90:175-181),
// the zero top and bottom rows of all eight fields, then DAMP_VELOCITY
template <typename T>
__global__ void mhd8_rhs_kernel(const MhdArgs A, const T* __restrict__ bg, const T* __restrict__ work,
                                const T* __restrict__ pab, const T* __restrict__ pml, T* __restrict__ spml, T beta,
                                int hs, const T* __restrict__ gz, const T* __restrict__ zt, int damp,
                                T* __restrict__ scr, SlotClock clk, int src_mode, const T* __restrict__ planes,
                                long long plane_ss, int L, const double* __restrict__ series, int nseries, int ksrc) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= A.N) return;
    const int s = blockIdx.y;
    const int k = (int)(t / A.NP);
    const long long q = t - (long long)k * A.NP;
    const T* w = work + (long long)s * V8_COUNT * A.N;
    auto W = [&](int f) { return w[(long long)f * A.N + t]; };
    auto B = [&](int f) { return bg[(long long)f * A.N + t]; };
    const T gpz = pml_bottom<T>(A, t, s, PV_P, W(V8_GPZ), pab, pml, spml, beta, hs);
    const T dvzdz = pml_bottom<T>(A, t, s, PV_VZ, W(V8_DVZDZ), pab, pml, spml, beta, hs);
    const T dzf2 = pml_bottom<T>(A, t, s, PV_IBX, W(V8_DZF2), pab, pml, spml, beta, hs);
    const T dzf1 = pml_bottom<T>(A, t, s, PV_IBY, W(V8_DZF1), pab, pml, spml, beta, hs);
    const T dzbx = pml_bottom<T>(A, t, s, PV_DZBX, W(V8_DZBX), pab, pml, spml, beta, hs);
    const T dzby = pml_bottom<T>(A, t, s, PV_DZBY, W(V8_DZBY), pab, pml, spml, beta, hs);
    const T rbx = W(V8_DYF3) - dzf2;
    const T rby = -W(V8_DXF3) + dzf1;
    const T rbz = W(V8_DXF2) - W(V8_DYF1);
    const T div = W(V8_DVXDX) + W(V8_DVYDY) + dvzdz;
    const T cbx = W(V8_DYBZ) - dzby;
    const T cby = -W(V8_DXBZ) + dzbx;
    const T cbz = W(V8_DXBY) - W(V8_DYBX);
    const T rho = W(V8_T0), vx = W(V8_T1), vy = W(V8_T2), vz = W(V8_T3);
    const T bx = W(V8_T5), by = W(V8_T6), bz = W(V8_T7);
    const T rcont = -B(MB_GR0X) * vx - B(MB_GR0Y) * vy - B(MB_GR0Z) * vz - B(MB_RHO0) * div;
    const T rp = -B(MB_C2RHO0) * div - vx * B(MB_GP0X) - vy * B(MB_GP0Y) - vz * B(MB_GP0Z);
    const T box = B(MB_BOX), boy = B(MB_BOY), boz = B(MB_BOZ), ri = B(MB_RHOINV);
    T f1 = cby * boz - cbz * boy, f2 = cbz * box - cbx * boz, f3 = cbx * boy - cby * box;
    T rvx = -ri * (W(V8_GPX) - f1);
    T rvy = -ri * (W(V8_GPY) - f2);
    T rvz = -ri * (gpz - f3);
    const T cbox = B(MB_CBOX), cboy = B(MB_CBOY), cboz = B(MB_CBOZ);
    f1 = cboy * bz - cboz * by; f2 = cboz * bx - cbox * bz; f3 = cbox * by - cboy * bx;
    rvx = rvx + ri * f1;
    rvy = rvy + ri * f2;
    rvz = rvz + ri * f3;
    rvz = rvz - ri * rho * gz[k];
    if (src_mode != 0 && abs(k - ksrc) <= 4) {
        const int tl = *clk.time - clk.t0[s];
        if (slot_src_on(clk, tl)) {
            const T* pl = planes + (long long)s * plane_ss + q;
            T F = (T)0;
            if (src_mode == 1) {
                const T wt = (tl < nseries) ? (T)series[(long long)s * nseries + tl] : (T)0;
                F = wt * pl[0];
            } else {
                for (int l = 0; l < 7; ++l) {
                    int id;
                    const double wl = lagrange_weight(clk, tl, L, l, &id);
                    if (id >= 0) F = F + (T)wl * pl[(long long)id * A.NP];
                }
            }
            rvz = rvz + F * zt[ZT_SRCDEP * A.nz + k];
        }
    }
    T out[8] = {rcont, rvx, rvy, rvz, rp, rbx, rby, rbz};
    if (k == 0 || k == A.nz - 1) {
        #pragma unroll
        for (int f = 0; f < 8; ++f) out[f] = (T)0;
    }
    if (damp) {
        out[1] = out[1] - W(V8_DMX);
        out[2] = out[2] - W(V8_DMY);
        out[3] = out[3] - W(V8_DMZ);
    }
    T* ss = scr + (long long)s * 8 * A.FS;
    #pragma unroll
    for (int f = 0; f < 8; ++f) ss[f * A.FS + t] = out[f];
}

template <typename T>
int mhd8_stage(sparc_ctx* c, T beta, int hs) {
    MhdState& m = *c->mhd;
    const int S = c->active_n, nz = c->nz;
    MhdArgs A;
    A.N = c->N; A.NP = c->NP; A.FS = 2 * c->fs; A.nz = nz; A.nb = c->P.npmlbot; A.nt = c->P.npmltop;
    A.nzpml = std::max(c->nzpml, 1);
    A.S = S;
    A.both = 1;
    A.nf = 8;
    T* work = (T*)m.work;
    const T* zt = (const T*)c->zt;
    const long long N = c->N, fst = (long long)V8_COUNT * N;
    const dim3 g(nb256(N), S);
    auto Wp = [&](int s, int f) { return work + ((size_t)s * V8_COUNT + f) * N; };
    int rc;
    mhd8_temp_kernel<T><<<g, 256, 0, c->stream>>>(A, (const T*)c->a, (const T*)c->scr, beta, hs, (const T*)m.bg, work);
    c->launches++;
    CKL();
    // the six ddxyz calls (pml.f90:106-116), all with bc 1; x and y per
    // source, z batched over the sources
    static const int xs[6][2] = {{V8_T1, V8_DVXDX}, {V8_F3, V8_DXF3}, {V8_T4, V8_GPX},
                                 {V8_F2, V8_DXF2}, {V8_T6, V8_DXBY}, {V8_T7, V8_DXBZ}};
    static const int ys[6][2] = {{V8_T2, V8_DVYDY}, {V8_T4, V8_GPY}, {V8_F3, V8_DYF3},
                                 {V8_T7, V8_DYBZ}, {V8_T5, V8_DYBX}, {V8_F1, V8_DYF1}};
    static const int zs[6][2] = {{V8_T3, V8_DVZDZ}, {V8_F1, V8_DZF1}, {V8_F2, V8_DZF2},
                                 {V8_T5, V8_DZBX}, {V8_T4, V8_GPZ}, {V8_T6, V8_DZBY}};
    for (int d = 0; d < 6; ++d) {
        for (int s = 0; s < S; ++s)
            if ((rc = ddx_launch<T>(c, Wp(s, xs[d][0]), Wp(s, xs[d][1]), nz)) ||
                (rc = ddy_launch<T>(c, Wp(s, ys[d][0]), Wp(s, ys[d][1]), nz)))
                return rc;
        if ((rc = ddz_launch<T>(c, zt, Wp(0, zs[d][0]), Wp(0, zs[d][1]), 1, S, fst))) return rc;
    }
    // DAMP_VELOCITY (damping.f90:125-159) of v_x, v_y, v_z
    const bool damp = c->P.damp_waves != 0;
    if (damp) {
        typedef typename CplxOf<T>::type CT;
        for (int s = 0; s < S; ++s)
            for (int q = 0; q < 3; ++q) {
                c->launches += fft_filter_phys<T>(Wp(s, V8_T1 + q), Wp(s, V8_DMX + q), (CT*)m.spec, (CT*)c->tmp,
                                                  c->P.nx, c->P.ny, nz, c->tw_x, c->tw_y, c->stream,
                                                  (const T*)c->pt + (size_t)PT_DAMP * c->M);
            }
        CKL();
    }
    SlotClock clk;
    memset(&clk, 0, sizeof(clk));
    clk.t0 = c->d_t0; clk.time = c->d_time; clk.freq = c->freq_filtering; clk.two_d = 0;
    clk.gate = c->forcing_length * c->cadforcing_step; clk.num_steps = c->num_steps;
    clk.ts = R4(c->P.timestep); clk.cad = R4(c->P.cadforcing);
    const int ksrc = (c->P.src_k > 0 ? c->P.src_k : c->e_rad) - 1;
    mhd8_rhs_kernel<T><<<g, 256, 0, c->stream>>>(A, (const T*)m.bg, work, (const T*)m.pab, (const T*)m.pml,
                                                  (T*)m.spml, beta, hs, (const T*)m.g, zt, damp ? 1 : 0,
                                                  (T*)c->scr, clk, c->src_mode, (const T*)c->planes,
                                                  (long long)c->src_L * c->NP, c->src_L, c->series, c->nseries,
                                                  ksrc);
    c->launches++;
    CKL();
    return SPARC_OK;
}

}  // namespace

namespace {

template <typename T>
int mhd_stage(sparc_ctx* c, T beta, int hs) {
    MhdState& m = *c->mhd;
    const int S = c->active_n, nz = c->nz;
    MhdArgs A;
    A.N = c->N; A.NP = c->NP; A.FS = 2 * c->fs; A.nz = nz; A.nb = c->P.npmlbot; A.nt = c->P.npmltop;
    A.nzpml = std::max(c->nzpml, 1);
    A.S = S;
    A.both = 0;
    A.nf = 6;
    T* a = (T*)c->a;
    T* scr = (T*)c->scr;
    T* bg = (T*)m.bg;
    T* work = (T*)m.work;
    const T* pab = (const T*)m.pab;
    T* pml = (T*)m.pml;
    T* spml = (T*)m.spml;
    const T* zt = (const T*)c->zt;
    const long long N = c->N;
    const dim3 g(nb256(N), S);
    auto Wp = [&](int s, int f) { return work + ((size_t)s * MW_COUNT + f) * N; };
    int rc;
    // independent derivatives of a group run on the second stream (side)
    // while the rest run on the context's stream; join before their consumer
    auto fork = [&]() -> int {
        CK(cudaEventRecord(m.evf, c->stream));
        CK(cudaStreamWaitEvent(m.s2, m.evf, 0));
        return SPARC_OK;
    };
    auto join = [&]() -> int {
        CK(cudaEventRecord(m.evj, m.s2));
        CK(cudaStreamWaitEvent(c->stream, m.evj, 0));
        return SPARC_OK;
    };
    auto side = [&](auto&& f) -> int {
        cudaStream_t s0 = c->stream;
        c->stream = m.s2;
        const int r = f();
        c->stream = s0;
        return r;
    };
    const long long wst = (long long)MW_COUNT * N;
    mhd_temp_kernel<T><<<g, 256, 0, c->stream>>>(A, a, scr, beta, hs, bg, work);
    c->launches++;
    CKL();
    // DAMP_VELOCITY (damping.f90:125-159) through the normalised 2-D transforms;
    // it needs only the temporaries, so its terms are ready for the RHS kernel
    const bool damp = c->P.damp_waves != 0;
    // div: ddxyz(xi_x, xi_y, xi_z, bc 1); d/dy and d/dz beside the damping
    // transforms and d/dx
    if ((rc = fork())) return rc;
    if ((rc = side([&]() -> int {
             for (int s = 0; s < S; ++s)
                 if (int r = ddy_launch<T>(c, Wp(s, MW_T1), Wp(s, MW_DY), nz)) return r;
             return ddz_launch<T>(c, zt, Wp(0, MW_T2), Wp(0, MW_DZ), 1, S, wst);
         })))
        return rc;
    if (damp) {
        typedef typename CplxOf<T>::type CT;
        for (int s = 0; s < S; ++s)
            for (int q = 0; q < 3; ++q) {
                c->launches += fft_filter_phys<T>(Wp(s, MW_T3 + q), Wp(s, MW_DMX + q), (CT*)m.spec, (CT*)c->tmp,
                                                  c->P.nx, c->P.ny, nz, c->tw_x, c->tw_y, c->stream,
                                                  (const T*)c->pt + (size_t)PT_DAMP * c->M);
            }
        CKL();
    }
    for (int s = 0; s < S; ++s)
        if ((rc = ddx_launch<T>(c, Wp(s, MW_T0), Wp(s, MW_DX), nz))) return rc;
    if ((rc = join())) return rc;
    mhd_div_kernel<T><<<g, 256, 0, c->stream>>>(A, bg, work, pab, pml, spml, beta, hs);
    c->launches++;
    CKL();
    // grad p: ddxyz(p, bc 0) and psi_p
    if ((rc = fork())) return rc;
    if ((rc = side([&]() -> int {
             for (int s = 0; s < S; ++s)
                 if (int r = ddy_launch<T>(c, Wp(s, MW_P), Wp(s, MW_GPY), nz)) return r;
             return ddz_launch<T>(c, zt, Wp(0, MW_P), Wp(0, MW_GPZ), 0, S, wst);
         })))
        return rc;
    for (int s = 0; s < S; ++s)
        if ((rc = ddx_launch<T>(c, Wp(s, MW_P), Wp(s, MW_GPX), nz))) return rc;
    if ((rc = join())) return rc;
    // induction: ddxyz(flux3, by, flux3, bx, flux2, dzflux2); ddxyz(flux2, bz, flux1, flux3, flux1, dzflux1).
    // d/dy(flux1) overwrites flux3, so it follows the join, after both reads of flux3
    if ((rc = fork())) return rc;
    if ((rc = side([&]() -> int {
             for (int s = 0; s < S; ++s)
                 if (int r = ddy_launch<T>(c, Wp(s, MW_F3), Wp(s, MW_BX), nz)) return r;
             if (int r = ddz_launch<T>(c, zt, Wp(0, MW_F2), Wp(0, MW_DZF2), 1, S, wst)) return r;
             return ddz_launch<T>(c, zt, Wp(0, MW_F1), Wp(0, MW_DZF1), 1, S, wst);
         })))
        return rc;
    for (int s = 0; s < S; ++s)
        if ((rc = ddx_launch<T>(c, Wp(s, MW_F3), Wp(s, MW_BY), nz)) || (rc = ddx_launch<T>(c, Wp(s, MW_F2), Wp(s, MW_BZ), nz)))
            return rc;
    if ((rc = join())) return rc;
    for (int s = 0; s < S; ++s)
        if ((rc = ddy_launch<T>(c, Wp(s, MW_F1), Wp(s, MW_F3), nz))) return rc;
    mhd_b_kernel<T><<<g, 256, 0, c->stream>>>(A, work, pab, pml, spml, beta, hs);
    c->launches++;
    CKL();
    // curl b: ddxyz(by, curlbz, bz, curlbx, bx, dzbx); ddxyz(bz, curlby, bx, flux1, by, dzby)
    if ((rc = fork())) return rc;
    if ((rc = side([&]() -> int {
             for (int s = 0; s < S; ++s)
                 if (int r = ddy_launch<T>(c, Wp(s, MW_BZ), Wp(s, MW_CBX), nz)) return r;
             for (int s = 0; s < S; ++s)
                 if (int r = ddy_launch<T>(c, Wp(s, MW_BX), Wp(s, MW_F1), nz)) return r;
             return ddz_launch<T>(c, zt, Wp(0, MW_BY), Wp(0, MW_DZBY), 1, S, wst);
         })))
        return rc;
    for (int s = 0; s < S; ++s)
        if ((rc = ddx_launch<T>(c, Wp(s, MW_BY), Wp(s, MW_CBZ), nz)) || (rc = ddx_launch<T>(c, Wp(s, MW_BZ), Wp(s, MW_CBY), nz)))
            return rc;
    if ((rc = ddz_launch<T>(c, zt, Wp(0, MW_BX), Wp(0, MW_DZBX), 1, S, wst))) return rc;
    if ((rc = join())) return rc;
    SlotClock clk;
    memset(&clk, 0, sizeof(clk));
    clk.t0 = c->d_t0; clk.time = c->d_time; clk.freq = c->freq_filtering; clk.two_d = 0;
    clk.gate = c->forcing_length * c->cadforcing_step; clk.num_steps = c->num_steps;
    clk.ts = R4(c->P.timestep); clk.cad = R4(c->P.cadforcing);
    mhd_rhs_kernel<T><<<g, 256, 0, c->stream>>>(A, bg, work, pab, pml, spml, beta, hs, (const T*)m.g,
                                                 (const T*)m.sponge, scr, damp ? 1 : 0, clk, c->src_mode,
                                                 (const T*)c->planes, (long long)c->src_L * c->NP, c->src_L,
                                                 c->series, c->nseries, m.plane, (const T*)m.dw);
    c->launches++;
    CKL();
    return SPARC_OK;
}

template <typename T>
int mhd_steps_t(sparc_ctx* c, int nsteps) {
    MhdState& m = *c->mhd;
    typedef typename CplxOf<T>::type CT;
    MhdArgs A;
    A.N = c->N; A.NP = c->NP; A.FS = 2 * c->fs; A.nz = c->nz; A.nb = c->P.npmlbot; A.nt = c->P.npmltop;
    A.nzpml = std::max(c->nzpml, 1);
    A.S = c->active_n;
    A.both = (c->P.option == 18 || c->P.option == 8);
    A.nf = c->nf;
    const int S = c->active_n;
    for (int it = 0; it < nsteps; ++it) {
        int rc;
        const bool two_d = (c->P.option == 18);
        for (int rk = 0; rk < 5; ++rk) {
            const T beta = (T)c->betas[rk];
            const int hs = rk > 0 ? 1 : 0;
            rc = two_d ? mhd2d_stage<T>(c, beta, hs)
                       : (c->P.option == 8 ? mhd8_stage<T>(c, beta, hs) : mhd_stage<T>(c, beta, hs));
            if (rc) return rc;
        }
        // update + z filter on all dimfive fields (step.f90:114-116, FILTER_VARS_3D)
        mhd_update_kernel<T><<<dim3((unsigned)((c->NP + 127) / 128), c->nf * S), 128, 0, c->stream>>>(
            A, (T*)c->a, (const T*)c->scr, (T)c->deltat, two_d ? 1 : 0);
        const long long npv = (long long)S * PV_COUNT * A.nzpml * c->NP;
        mhd_pml_update_kernel<T><<<nb256(npv), 256, 0, c->stream>>>((T*)m.pml, (const T*)m.spml, (T)c->deltat, npv);
        c->launches += 2;
        CKL();
        // horizontal filter every freq_filtering steps of each slot's clock:
        // 3-D on fields 1..5 when mod(time, 30) = 0 (physics.f90:791-830),
        // 2-D on all six when mod(time+1, 30) = 0 (physics2d.f90:566-584)
        for (int s = 0; s < S; ++s) {
            const int tl = c->time - c->t0[s];
            if (tl < 0 || (two_d ? (tl + 1) : tl) % c->freq_filtering != 0) continue;
            for (int f = 0; f < (two_d ? 6 : 5); ++f) {
                T* fp = (T*)c->a + ((size_t)s * c->nf + f) * 2 * c->fs;
                c->launches += fft_filter_phys<T>(fp, fp, (CT*)m.spec, (CT*)c->tmp, c->P.nx, c->P.ny, c->nz, c->tw_x,
                                                  c->tw_y, c->stream, (const T*)c->pt + (size_t)PT_HF * c->M);
            }
            CKL();
        }
        if (c->rec_on) {
            mhd_record_kernel<T><<<dim3(nb256(c->NP), S), 256, 0, c->stream>>>(
                (const T*)c->a, (T*)c->rec, c->d_t0, c->d_time, c->steps, c->rec_max, 2 * c->fs, c->NP,
                (long long)c->rec_max * 2 * c->M, m.plane_obs, c->nf, c->P.option == 8 ? 3 : 5);
            c->launches++;
            CKL();
        }
        launch_tick(c->d_time, c->stream);
        c->launches++;
        CKL();
        c->time++;
    }
    return SPARC_OK;
}

}  // namespace

int mhd_steps(sparc_ctx* c, int nsteps) {
    if (!c->mhd || !c->mhd->have_bg)
        return fail(c, SPARC_ESTATE, c->P.option == 18 ? "option 18 needs sparc_gpu_set_mhd2d_background"
                                                        : "options 8 and 10 need sparc_gpu_set_mhd_background");
    return c->f32 ? mhd_steps_t<float>(c, nsteps) : mhd_steps_t<double>(c, nsteps);
}

// ---- sensitivity kernels of the 2-D MHD form (option 18) ---------------------

namespace {

// ddzkern: DBYD2 * stretch, then FILTER_VAR_Z (kernels.f90:609-621)
template <typename T>
int ddzk_launch(sparc_ctx* c, const T* zt, const T* in, T* out, int bc) {
    int rc = ddz_launch<T>(c, zt, in, out, bc, 1, 0);
    if (rc) return rc;
    zfilter_phys_kernel<T><<<dim3(nb256(c->NP), 1), 256, 0, c->stream>>>(out, c->NP, c->nz, 0);
    c->launches++;
    CKL();
    return SPARC_OK;
}

// the seven physical fields of a kernel snapshot of sources s0..s0+G-1 (the
// layout of the quiet path's store): forward div(xi) (COMPUTE_DIV), acc =
// scr(v) (3), xi (3); adjoint div(v), v (3), grad(v_z grav) (3)
template <typename T>
int mhd2d_derive_t(sparc_ctx* c, int s0, int G, bool adjoint, T* out, long long ofs) {
    MhdState& m = *c->mhd;
    const long long N = c->N, fs2 = 2 * c->fs;
    const T* zt = (const T*)c->zt;
    T* sc = (T*)m.work + (size_t)MW_P * N;      // scratch: work fields of slot 0
    T* sc2 = (T*)m.work + (size_t)MW_R * N;
    int rc;
    for (int g = 0; g < G; ++g) {
        const int s = s0 + g;
        auto A = [&](int f) { return (T*)c->a + ((size_t)s * c->nf + f) * fs2; };
        auto S = [&](int f) { return (T*)c->scr + ((size_t)s * c->nf + f) * fs2; };
        auto O = [&](int f) { return out + (size_t)f * ofs + (size_t)g * N; };
        const int fx = adjoint ? 3 : 0;
        if ((rc = ddx_launch<T>(c, A(fx), O(0), c->nz)) || (rc = ddzk_launch<T>(c, zt, A(fx + 2), sc, 1))) return rc;
        add_kernel<T><<<nb256(N), 256, 0, c->stream>>>(O(0), sc, N);
        for (int q = 0; q < 3; ++q) {
            CK(cudaMemcpyAsync(O(1 + q), adjoint ? A(3 + q) : S(3 + q), N * sizeof(T), cudaMemcpyDeviceToDevice,
                               c->stream));
            if (!adjoint) CK(cudaMemcpyAsync(O(4 + q), A(q), N * sizeof(T), cudaMemcpyDeviceToDevice, c->stream));
        }
        if (adjoint) {
            // grad(v_z grav) (kernels.f90:299-304)
            zscale_kernel<T><<<nb256(N), 256, 0, c->stream>>>(sc2, A(5), zt + (size_t)ZT_GRAW * c->nz, c->NP, N);
            if ((rc = ddx_launch<T>(c, sc2, O(4), c->nz)) || (rc = ddzk_launch<T>(c, zt, sc2, O(6), 1))) return rc;
            CK(cudaMemsetAsync(O(5), 0, N * sizeof(T), c->stream));
        }
        c->launches += adjoint ? 3 : 1;
        CKL();
    }
    return SPARC_OK;
}

// the y-only products of the MAGNETIC_KERNELS block in 2-D (B0 = (Bx, 0, Bz),
// curl B0 = (0, cby, 0), d/dy = 0): ty = (xi x B0)_y, uy = (v x B0)_y,
// (wx, wz) = v x curl B0, vy = (B0 x xi div v)_y
template <typename T>
__global__ void kb_products_kernel(const T* __restrict__ fxx, const T* __restrict__ fxz, const T* __restrict__ avx,
                                   const T* __restrict__ avz, const T* __restrict__ dA, const T* __restrict__ box,
                                   const T* __restrict__ boz, const T* __restrict__ cby, T* __restrict__ ty,
                                   T* __restrict__ uy, T* __restrict__ wx, T* __restrict__ wz, T* __restrict__ vy,
                                   long long n) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    ty[t] = box[t] * fxz[t] - fxx[t] * boz[t];
    uy[t] = box[t] * avz[t] - avx[t] * boz[t];
    wx[t] = -(avz[t] * cby[t]);
    wz[t] = avx[t] * cby[t];
    const T tx = fxx[t] * dA[t], tz = fxz[t] * dA[t];
    vy[t] = tx * boz[t] - box[t] * tz;
}

// fb = curl(0, ty, 0) = (-ddzk ty, 0, d ty/dx); ab likewise from uy; t3y = (fb x v)_y
template <typename T>
__global__ void kb_curls_kernel(T* __restrict__ fbx, const T* __restrict__ fbz, T* __restrict__ abx,
                                const T* __restrict__ avx, const T* __restrict__ avz, T* __restrict__ t3y,
                                long long n) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const T bx = -fbx[t];
    fbx[t] = bx;
    abx[t] = -abx[t];
    t3y[t] = avx[t] * fbz[t] - bx * avz[t];
}

// kernelb += the six terms in the reference's order (kernels.f90:337-453)
template <typename T>
__global__ void kb_accum_kernel(double* __restrict__ kbx, double* __restrict__ kbz, const T* __restrict__ fxx,
                                const T* __restrict__ fxz, const T* __restrict__ avx, const T* __restrict__ avz,
                                const T* __restrict__ dA, const T* __restrict__ cby, const T* __restrict__ r1,
                                const T* __restrict__ r2, const T* __restrict__ u1, const T* __restrict__ u2,
                                const T* __restrict__ s1, const T* __restrict__ s2, const T* __restrict__ p1,
                                const T* __restrict__ p2, const T* __restrict__ q1, const T* __restrict__ q2,
                                long long n) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const T t2y = r1[t] - r2[t];                    // curl(curl(xi x B0))_y
    const T t4y = s1[t] - s2[t];                    // curl(curl(v x B0))_y
    const T sy = p1[t] - p2[t];                     // curl(v x curl B0)_y
    double x = kbx[t], z = kbz[t];
    x = x + (double)(-(avz[t] * t2y)); z = z + (double)(avx[t] * t2y);
    x = x + (double)(-u1[t]);          z = z + (double)u2[t];
    x = x + (double)(-(fxz[t] * t4y)); z = z + (double)(fxx[t] * t4y);
    x = x + (double)(sy * fxz[t]);     z = z + (double)(-(sy * fxx[t]));
    x = x + (double)(-(fxz[t] * cby[t]) * dA[t]);
    z = z + (double)((fxx[t] * cby[t]) * dA[t]);
    x = x + (double)(-q1[t]);          z = z + (double)q2[t];
    kbx[t] = x;
    kbz[t] = z;
}

template <typename T>
int mhd2d_kernel_b_t(sparc_ctx* c, const T* fst, long long sfs, const T* adj, long long afs, int s0, int G) {
    MhdState& m = *c->mhd;
    const long long N = c->N;
    const T* zt = (const T*)c->zt;
    T* w = (T*)m.work;                               // work fields of slot 0 as scratch
    auto Wf = [&](int i) { return w + (size_t)i * N; };
    T *ty = Wf(0), *uy = Wf(1), *wx = Wf(2), *wz = Wf(3), *vy = Wf(4), *fbx = Wf(5), *fbz = Wf(6), *abx = Wf(7);
    T *abz = Wf(8), *p1 = Wf(9), *p2 = Wf(10), *q1 = Wf(11), *q2 = Wf(12), *t3y = Wf(13), *r1 = Wf(14);
    T *r2 = Wf(15), *s1 = Wf(16), *s2 = Wf(17), *u1 = Wf(18), *u2 = Wf(19);
    const unsigned nb = nb256(N);
    int rc;
    for (int g = 0; g < G; ++g) {
        const T* fxx = fst + 4 * sfs + (size_t)g * N;
        const T* fxz = fst + 6 * sfs + (size_t)g * N;
        const T* dA = adj + (size_t)g * N;
        const T* avx = adj + afs + (size_t)g * N;
        const T* avz = adj + 3 * afs + (size_t)g * N;
        double* kb = m.kbacc + (size_t)(s0 + g) * 2 * N;
        kb_products_kernel<T><<<nb, 256, 0, c->stream>>>(fxx, fxz, avx, avz, dA, (const T*)m.kbox,
                                                         (const T*)m.bg + (size_t)MB_BOZ * N, (const T*)m.kcby, ty, uy,
                                                         wx, wz, vy, N);
        if ((rc = ddzk_launch<T>(c, zt, ty, fbx, 0)) || (rc = ddx_launch<T>(c, ty, fbz, c->nz)) ||
            (rc = ddzk_launch<T>(c, zt, uy, abx, 0)) || (rc = ddx_launch<T>(c, uy, abz, c->nz)) ||
            (rc = ddzk_launch<T>(c, zt, wx, p1, 0)) || (rc = ddx_launch<T>(c, wz, p2, c->nz)) ||
            (rc = ddzk_launch<T>(c, zt, vy, q1, 0)) || (rc = ddx_launch<T>(c, vy, q2, c->nz)))
            return rc;
        kb_curls_kernel<T><<<nb, 256, 0, c->stream>>>(fbx, fbz, abx, avx, avz, t3y, N);
        if ((rc = ddzk_launch<T>(c, zt, fbx, r1, 0)) || (rc = ddx_launch<T>(c, fbz, r2, c->nz)) ||
            (rc = ddzk_launch<T>(c, zt, abx, s1, 0)) || (rc = ddx_launch<T>(c, abz, s2, c->nz)) ||
            (rc = ddzk_launch<T>(c, zt, t3y, u1, 0)) || (rc = ddx_launch<T>(c, t3y, u2, c->nz)))
            return rc;
        kb_accum_kernel<T><<<nb, 256, 0, c->stream>>>(kb, kb + N, fxx, fxz, avx, avz, dA, (const T*)m.kcby, r1, r2,
                                                      u1, u2, s1, s2, p1, p2, q1, q2, N);
        c->launches += 3;
        CKL();
    }
    return SPARC_OK;
}

// kernel_b * scale for x and z, and the vector-potential kernel as the y
// component of CURL_KERN of (kernel_bx, 0, kernel_bz), in FP64
__global__ void kb_finish_kernel(double* __restrict__ out, const double* __restrict__ acc, double scale, int nsum,
                                 long long acc_ss, long long n) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    double x = 0, z = 0;
    for (int s = 0; s < nsum; ++s) {
        x += acc[s * acc_ss + t];
        z += acc[s * acc_ss + n + t];
    }
    out[t] = x * scale;
    out[n + t] = z * scale;
}

}  // namespace

int mhd2d_derive(sparc_ctx* c, int s0, int G, bool adjoint, void* out, long long ofs) {
    if (!c->mhd || c->P.option != 18) return fail(c, SPARC_EINVAL, "kernel snapshots of the MHD forms need option 18");
    return c->f32 ? mhd2d_derive_t<float>(c, s0, G, adjoint, (float*)out, ofs)
                  : mhd2d_derive_t<double>(c, s0, G, adjoint, (double*)out, ofs);
}

int mhd2d_kernel_b_reset(sparc_ctx* c) {
    MhdState& m = *c->mhd;
    if (!m.kbacc) {
        int rc = dalloc(c, (void**)&m.kbacc, (size_t)c->S * 2 * c->N * 8);
        if (rc) return rc;
    }
    CK(cudaMemsetAsync(m.kbacc, 0, (size_t)c->S * 2 * c->N * 8, c->stream));
    return SPARC_OK;
}

int mhd2d_kernel_b_accumulate(sparc_ctx* c, const void* fst, long long sfs, const void* adj, long long afs, int s0,
                              int G) {
    MhdState& m = *c->mhd;
    if (!m.kbacc) { int rc = mhd2d_kernel_b_reset(c); if (rc) return rc; }
    return c->f32 ? mhd2d_kernel_b_t<float>(c, (const float*)fst, sfs, (const float*)adj, afs, s0, G)
                  : mhd2d_kernel_b_t<double>(c, (const double*)fst, sfs, (const double*)adj, afs, s0, G);
}

int mhd2d_kernels_b(sparc_ctx* c, int src, int sum_slots, double* kbx, double* kbz, double* kpsi) {
    MhdState& m = *c->mhd;
    if (!m.kbacc) return fail(c, SPARC_ESTATE, "no B-field kernel accumulation yet");
    const long long N = c->N;
    // kernels.f90:498-514 (2-D: dimen = (diml 1e-8 xlength 1e-8 dimb)^-1)
    const double dimb = std::sqrt(4.0 * c->pi * c->dimc * c->dimc * c->dimrho);
    const double dimen = 1.0 / (c->diml * (double)1.0e-8f * R4(c->P.xlength) * (double)1.0e-8f * dimb);
    const double scale = (double)c->steps * R4(c->P.timestep) * dimen;
    double* out = nullptr;
    int rc = dalloc(c, (void**)&out, (size_t)4 * N * 8);
    if (rc) return rc;
    const double* acc = m.kbacc + (sum_slots ? 0 : (size_t)src * 2 * N);
    kb_finish_kernel<<<nb256(N), 256, 0, c->stream>>>(out, acc, scale, sum_slots ? c->S : 1, 2 * N, N);
    c->launches++;
    // psi kernel: ddzkern(kernel_bx, 0) - d kernel_bz/dx (FP64 multipliers)
    void* rx0 = m.rx;
    m.rx = m.rx64;
    rc = ddz_launch<double>(c, c->zt64, out, out + 2 * N, 0, 1, 0);
    if (!rc) {
        zfilter_phys_kernel<double><<<dim3(nb256(c->NP), 1), 256, 0, c->stream>>>(out + 2 * N, c->NP, c->nz, 0);
        rc = ddx_launch<double>(c, out + N, out + 3 * N, c->nz);
    }
    m.rx = rx0;
    if (!rc) {
        axpby_kernel<<<nb256(N), 256, 0, c->stream>>>(out + 2 * N, out + 2 * N, 1.0, out + 3 * N, -1.0, N);
        c->launches += 2;
        if (kbx) CK(cudaMemcpyAsync(kbx, out, N * 8, cudaMemcpyDeviceToHost, c->stream));
        if (kbz) CK(cudaMemcpyAsync(kbz, out + N, N * 8, cudaMemcpyDeviceToHost, c->stream));
        if (kpsi) CK(cudaMemcpyAsync(kpsi, out + 2 * N, N * 8, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
    }
    cudaFree(out);
    c->allocs.erase(std::remove(c->allocs.begin(), c->allocs.end(), (void*)out), c->allocs.end());
    c->dev_bytes -= (long long)4 * N * 8;
    return rc;
}

const double* mhd_kernel_c2(const sparc_ctx* c) { return (c->mhd && c->P.option == 18) ? c->mhd->kc2 : nullptr; }
const double* mhd_kernel_rho0(const sparc_ctx* c) { return (c->mhd && c->P.option == 18) ? c->mhd->krho : nullptr; }
