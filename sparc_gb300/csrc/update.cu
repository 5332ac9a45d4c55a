// Model update of an inversion iteration on the device (grad.py:158-301):
// Hessian preconditioning, the z filters, antisymmetrize, the reductions of
// the update direction and the line-search test models.  The x smoothing
// (filterx) runs through the FP64 transforms with a pencil multiplier.
//
// Element-wise kernels are grid-stride free (one thread per point); the z
// filters give one thread per (y, x) column, so a warp reads 32 adjacent
// points of each plane.  Reductions are two passes over a fixed grid, so
// the result does not depend on timing.
#include <cmath>

#include "update.cuh"

namespace {

constexpr int kRedBlocks = 1216;      // 8 CTAs per SM on 152 SMs
constexpr int kRedThreads = 256;
constexpr int kMaxTaps = 65;

unsigned nbk(long long n) { return (unsigned)((n + 255) / 256); }

struct Taps { double w[kMaxTaps]; };

__global__ void reduce_partial_kernel(double* part, const double* __restrict__ a, const double* __restrict__ b,
                                      long long n) {
    __shared__ double ss[kRedThreads], sa[kRedThreads], sm[kRedThreads];
    double s = 0.0, ma = 0.0, mx = -INFINITY;
    for (long long t = (long long)blockIdx.x * kRedThreads + threadIdx.x; t < n; t += (long long)gridDim.x * kRedThreads) {
        const double v = a[t];
        s = fma(v, b ? b[t] : v, s);
        ma = fmax(ma, fabs(v));
        mx = fmax(mx, v);
    }
    ss[threadIdx.x] = s; sa[threadIdx.x] = ma; sm[threadIdx.x] = mx;
    __syncthreads();
    for (int w = kRedThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            ss[threadIdx.x] += ss[threadIdx.x + w];
            sa[threadIdx.x] = fmax(sa[threadIdx.x], sa[threadIdx.x + w]);
            sm[threadIdx.x] = fmax(sm[threadIdx.x], sm[threadIdx.x + w]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[blockIdx.x] = ss[0];
        part[kRedBlocks + blockIdx.x] = sa[0];
        part[2 * kRedBlocks + blockIdx.x] = sm[0];
    }
}

__global__ void reduce_final_kernel(double* res, const double* __restrict__ part, int nb) {
    __shared__ double ss[kRedThreads], sa[kRedThreads], sm[kRedThreads];
    double s = 0.0, ma = 0.0, mx = -INFINITY;
    for (int t = threadIdx.x; t < nb; t += kRedThreads) {
        s += part[t];
        ma = fmax(ma, part[kRedBlocks + t]);
        mx = fmax(mx, part[2 * kRedBlocks + t]);
    }
    ss[threadIdx.x] = s; sa[threadIdx.x] = ma; sm[threadIdx.x] = mx;
    __syncthreads();
    for (int w = kRedThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            ss[threadIdx.x] += ss[threadIdx.x + w];
            sa[threadIdx.x] = fmax(sa[threadIdx.x], sa[threadIdx.x + w]);
            sm[threadIdx.x] = fmax(sm[threadIdx.x], sm[threadIdx.x + w]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) { res[0] = ss[0]; res[1] = sa[0]; res[2] = sm[0]; }
}

__global__ void hess_scale_kernel(double* hess, const double* __restrict__ rho_z, long long npix, long long n) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) hess[t] = hess[t] * rho_z[t / npix];
}

__global__ void hess_floor_kernel(double* hess, const double* __restrict__ hmax, long long n) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const double h = hess[t] / hmax[2];
    hess[t] = h < 5e-3 ? 5e-3 : h;
}

__global__ void divide_kernel(double* out, const double* a, const double* h, long long n) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) out[t] = a[t] / h[t];
}

// grad.py:63-96 with the planes its temp array never writes (4 and nz-1)
// left at zero and plane 0 kept
__global__ void filterz_smooth_kernel(double* __restrict__ out, const double* __restrict__ in, long long npix,
                                      int nz) {
    const long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= npix) return;
    const double c[6] = {0.75390625, 0.41015625, -0.234375, 0.087890625, -0.01953125, 0.001953125};
    auto A = [&](int k) { return in[(long long)k * npix + m]; };
    for (int k = 0; k < nz; ++k) {
        double v;
        if (k == 0) {
            v = A(0);
        } else if (k >= 5 && k <= nz - 6) {
            v = c[0] * A(k);
            for (int j = 1; j <= 5; ++j) v = v + 0.5 * c[j] * (A(k - j) + A(k + j));
        } else if ((k >= 1 && k <= 3) || (k >= nz - 5 && k <= nz - 2)) {
            v = 0.5 * (A(k - 1) + A(k + 1));
        } else {
            v = 0.0;
        }
        out[(long long)k * npix + m] = v;
    }
}

__global__ void gaussian_z_kernel(double* __restrict__ out, const double* __restrict__ in, long long npix, int nz,
                                  Taps taps, int r) {
    const long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= npix) return;
    const int period = 2 * nz;
    for (int k = 0; k < nz; ++k) {
        double acc = 0.0;
        for (int j = 0; j <= 2 * r; ++j) {
            int q = ((k - r + j) % period + period) % period;
            q = q < nz ? q : period - 1 - q;          // half-sample symmetric: d c b a | a b c d | d c b a
            acc = acc + taps.w[j] * in[(long long)q * npix + m];
        }
        out[(long long)k * npix + m] = acc;
    }
}

__global__ void antisym_kernel(double* out, const double* in, long long nrows, int nx) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nrows * nx) return;
    const long long row = t / nx;
    const int i = (int)(t - row * nx);
    out[t] = 0.5 * (in[t] - in[row * nx + (nx - 1 - i)]);
}

__global__ void axpy_c_kernel(double* out, const double* a, const double* b, double c, long long n) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) out[t] = a[t] + c * b[t];
}

__global__ void sub_kernel(double* out, const double* a, const double* b, long long n) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) out[t] = a[t] - b[t];
}

__global__ void test_model_kernel(double* out, const double* model, const double* u, const double* umax, double coef,
                                  long long n) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) out[t] = model[t] + coef * (u[t] / umax[1]);
}

}  // namespace

void launch_reduce(double* res, const double* a, const double* b, long long n, double* scratch, cudaStream_t s) {
    long long nb = (n + kRedThreads - 1) / kRedThreads;
    if (nb > kRedBlocks) nb = kRedBlocks;
    if (nb < 1) nb = 1;
    reduce_partial_kernel<<<(unsigned)nb, kRedThreads, 0, s>>>(scratch, a, b, n);
    reduce_final_kernel<<<1, kRedThreads, 0, s>>>(res, scratch, (int)nb);
}

void launch_precondition(double* hess, const double* rho_z, long long npix, int nz, double* scratch, cudaStream_t s) {
    const long long n = npix * nz;
    hess_scale_kernel<<<nbk(n), 256, 0, s>>>(hess, rho_z, npix, n);
    launch_reduce(scratch, hess, nullptr, n, scratch + 4, s);
    hess_floor_kernel<<<nbk(n), 256, 0, s>>>(hess, scratch, n);
}

void launch_divide(double* out, const double* a, const double* h, long long n, cudaStream_t s) {
    divide_kernel<<<nbk(n), 256, 0, s>>>(out, a, h, n);
}

void launch_filterz_smooth(double* out, const double* in, long long npix, int nz, cudaStream_t s) {
    filterz_smooth_kernel<<<nbk(npix), 256, 0, s>>>(out, in, npix, nz);
}

bool launch_gaussian_z(double* out, const double* in, long long npix, int nz, double sigma, cudaStream_t s) {
    // the taps of scipy's gaussian_filter1d: exp(-x^2 / 2 sigma^2), x = -r..r,
    // r = int(4 sigma + 0.5), scaled to sum 1
    const int r = (int)(4.0 * sigma + 0.5);
    if (2 * r + 1 > kMaxTaps || r < 0) return false;
    Taps taps = {};
    double sum = 0.0;
    for (int j = 0; j <= 2 * r; ++j) {
        const double x = j - r;
        taps.w[j] = std::exp(-0.5 / (sigma * sigma) * (x * x));
        sum += taps.w[j];
    }
    for (int j = 0; j <= 2 * r; ++j) taps.w[j] = taps.w[j] / sum;
    gaussian_z_kernel<<<nbk(npix), 256, 0, s>>>(out, in, npix, nz, taps, r);
    return true;
}

void launch_antisymmetrize(double* out, const double* in, long long nrows, int nx, cudaStream_t s) {
    antisym_kernel<<<nbk(nrows * nx), 256, 0, s>>>(out, in, nrows, nx);
}

void launch_axpy_c(double* out, const double* a, const double* b, double c, long long n, cudaStream_t s) {
    axpy_c_kernel<<<nbk(n), 256, 0, s>>>(out, a, b, c, n);
}

void launch_sub(double* out, const double* a, const double* b, long long n, cudaStream_t s) {
    sub_kernel<<<nbk(n), 256, 0, s>>>(out, a, b, n);
}

void launch_test_model(double* out, const double* model, const double* u, const double* umax, double coef, long long n,
                       cudaStream_t s) {
    test_model_kernel<<<nbk(n), 256, 0, s>>>(out, model, u, umax, coef, n);
}
