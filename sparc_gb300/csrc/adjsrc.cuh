// Adjoint source of a 2-D run (ADJOINT_SOURCE_FILT, driver.f90:1262-1686).
#pragma once
#include <string>

#include <cuda_runtime.h>

struct AdjSrcArgs {
    double x00;            // master pixel x (Mm)
    double t1, dt;         // first output time and cadence, minutes
    int have_ridge[3];     // params.0 (f), params.1 (p1), params.2 (band-passed phase-speed set)
    double ridge[3][3];    // mindist (Mm), maxdist (Mm), window (min)
    int have_band[2];      // filter.params.0 / .1
    double band[2][2];     // left, right corner (mHz)
    int linesearch;        // windows of modes 0, 1 read from `windows` instead of chosen
};

// acc_dev: synthetic surface v_z on the device, (nt, nx) FP64; dat_host: the
// observed data, (nt, nx); windows: [2][nx][2] (lef, rig, 1-based; 0 = no
// measurement), written unless a.linesearch; adj_host: (nt, nx).  Returns 0,
// 1 (bad input, `why` set) or 2 (CUDA failure).
int adjsrc_compute(cudaStream_t s, const double* acc_dev, const double* dat_host, int nt, int nx, double xlength,
                   double outputcad, const AdjSrcArgs& a, int* windows, double* adj_host, double* misfit,
                   int* nmeas, std::string& why);

// MISFIT_ALL (driver.f90:1702-2076): for the bands 2-3.5, 3.5-4.5, 4.5-6 mHz
// the three sets of ADJOINT_SOURCE_FILT with MISFIT_ALL's ridge speeds and
// arrival polynomial; misfit[band][set] = 0.5 sum tau^2, nmeas[band][set];
// windows: [3][2][nx][2] (the band's sets 0 and 1; windows.all.N).
int misfit_all_compute(cudaStream_t s, const double* acc_dev, const double* dat_host, int nt, int nx, double xlength,
                       double outputcad, const AdjSrcArgs& a, int* windows, double* misfit, int* nmeas,
                       std::string& why);
