// Model update of an inversion iteration (grad.py:158-301), device parts.
// All arrays are FP64, (nz, npix) with npix = ny * nx.
#pragma once
#include <cuda_runtime.h>

// partial-sum slots a reduction needs in its scratch (doubles)
constexpr int kReduceScratch = 3 * 1216 + 4;

// res[0] = sum a*b (b null: sum a*a), res[1] = max |a|, res[2] = max a, summed
// in a fixed order (two passes); scratch holds kReduceScratch doubles
void launch_reduce(double* res, const double* a, const double* b, long long n, double* scratch, cudaStream_t s);
// hess = max(hess rho_z[k] / max(hess rho_z), 5e-3) in place; scratch as
// launch_reduce's plus 4
void launch_precondition(double* hess, const double* rho_z, long long npix, int nz, double* scratch,
                         cudaStream_t s);
// out = a / h
void launch_divide(double* out, const double* a, const double* h, long long n, cudaStream_t s);
// filterz 'smooth' (grad.py:63-96) of in into out
void launch_filterz_smooth(double* out, const double* in, long long npix, int nz, cudaStream_t s);
// scipy's gaussian_filter1d along z, mode 'reflect' (grad.py:106-107);
// false if the stencil (2 int(4 sigma + 0.5) + 1 taps) is over 65 taps
bool launch_gaussian_z(double* out, const double* in, long long npix, int nz, double sigma, cudaStream_t s);
// out = 0.5 (a - a reversed along x), rows of nx
void launch_antisymmetrize(double* out, const double* in, long long nrows, int nx, cudaStream_t s);
// out = a + c b
void launch_axpy_c(double* out, const double* a, const double* b, double c, long long n, cudaStream_t s);
// out = a - b
void launch_sub(double* out, const double* a, const double* b, long long n, cudaStream_t s);
// out = model + coef (u / umax[0])
void launch_test_model(double* out, const double* model, const double* u, const double* umax, double coef,
                       long long n, cudaStream_t s);
