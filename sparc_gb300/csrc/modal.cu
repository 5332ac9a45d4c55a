// Time-stepping kernels on the spectral-column state (see internal.cuh).
//
// One thread owns one horizontal Fourier mode m of one source and walks its
// z-pencil.  Loads and stores of a warp touch 32 consecutive modes of one
// z-plane, so every global access is a coalesced 16 B (FP64) / 8 B (FP32)
// per-lane transaction.
//
// stage_kernel = one RK stage of MP_QUIET_PML_3D_DISPL (displacement.f90:482-658)
// or MP_QUIET_PML_2D_DISPL (physics2d.f90:948-1105), with temp = a + beta*scr
// (step.f90:52-71) formed on the fly.  Four sweeps over z:
//   S1 (up)   compact RHS of d(xi_z)/dz and forward elimination -> y
//   S2 (down) back substitution, stretch, PML psi_vz, div, p', rho'; writes the
//             horizontal RHS (v_x, v_y, xi_x, xi_y) point-wise
//   S3 (up)   compact RHS of dp'/dz and forward elimination -> y
//   S4 (down) back substitution, stretch, PML psi_p, RHS v_z (+source, damping),
//             RHS xi_z, boundary zeroing
// update_kernel = a += dt*scr, pmlvars += dt*scrpml (step.f90:114-116) fused with
// the z filter and, every freq_filtering steps, the horizontal spectral filter
// (FILTER_VARS_3D physics.f90:741-833 / FILTER_VARS_2D physics2d.f90:514-588).
#include "internal.cuh"

template <typename T>
__global__ void __launch_bounds__(128) stage_kernel(const StageArgs<T> A) {
    typedef typename CplxOf<T>::type CT;
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= A.M) return;
    const int s = blockIdx.y;
    const int nz = A.nz;
    const long long M = A.M, fs = A.fs;
    CT* __restrict__ a = A.a + (long long)s * 6 * fs + m;
    CT* __restrict__ scr = A.scr + (long long)s * 6 * fs + m;
    CT* __restrict__ pml = A.pml + (long long)s * 2 * A.ps + m;
    CT* __restrict__ spml = A.scrpml + (long long)s * 2 * A.ps + m;
    CT* __restrict__ y = A.ybuf + (long long)s * fs + m;
    CT* __restrict__ pb = A.pbuf + (long long)s * fs + m;
    CT* __restrict__ rb = A.rbuf + (long long)s * fs + m;
    const T* __restrict__ zt = A.zt;
    const T kx = __ldg(&A.pt[PT_KX * M + m]);
    const T ky = __ldg(&A.pt[PT_KY * M + m]);
    const T gd = A.damp ? __ldg(&A.pt[PT_DAMP * M + m]) : (T)0;
    const T beta = A.beta;
    const bool hs = A.has_scr != 0;
    const bool opt3d = (A.option == 4);
    const int nb = A.npmlbot, nt = A.npmltop;
    const int bcx = opt3d ? 1 : 3, bcp = opt3d ? 0 : 2;

    auto temp = [&](int f, int j) -> CT {
        long long o = f * fs + (long long)j * M;
        CT v = a[o];
        if (hs) v = v + beta * scr[o];
        return v;
    };
    auto pmlidx = [&](int j) -> int { return j < nb ? j : (j >= nz - nt ? nb + (j - (nz - nt)) : -1); };

    // ---------------- S1: d(xi_z)/dz, forward elimination -------------------
    CT top = czero<CT>();
    if (!opt3d) {   // physics2d.f90:960: dxizdz(nz) = -dxixdx(nz) * unstretch(nz)
        CT xx = temp(0, nz - 1);
        top = -(imul(kx, xx) * __ldg(&zt[ZT_UNSTRETCH * nz + nz - 1]));
    }
    compact_forward<CT, T>(nz, bcx, [&](int j) { return temp(2, j); }, czero<CT>(), top,
                           zt + (ZT_TH + 3 * bcx) * nz, zt + (ZT_TH + 3 * bcx + 1) * nz, A.cc, y, M);

    // ---------------- S2: back substitution, div, p', rho', horizontal RHS ---
    {
        const T* gam = zt + (ZT_TH + 3 * bcx + 2) * nz;
        CT ud = y[(long long)(nz - 1) * M];
        for (int j = nz - 1; j >= 0; --j) {
            if (j < nz - 1) ud = y[(long long)j * M] - __ldg(&gam[j + 1]) * ud;
            CT dz = ud * __ldg(&zt[ZT_STRETCH * nz + j]);
            int ip = pmlidx(j);
            if (ip >= 0) {
                long long o = (long long)ip * M;
                CT psi = pml[o];
                if (hs) psi = psi + beta * spml[o];
                spml[o] = __ldg(&zt[ZT_AZ * nz + j]) * dz + __ldg(&zt[ZT_BZ * nz + j]) * psi;
                dz = dz + psi;
            }
            CT xx = temp(0, j), xz = temp(2, j);
            CT div;
            if (opt3d) div = imul(kx, xx) + imul(ky, temp(1, j)) + dz;
            else div = imul(kx, xx) + dz;
            CT p = -__ldg(&zt[ZT_C2RHO0 * nz + j]) * div - __ldg(&zt[ZT_GRADP0 * nz + j]) * xz;
            CT r = -__ldg(&zt[ZT_RHO0 * nz + j]) * div - __ldg(&zt[ZT_GRADRHO0 * nz + j]) * xz;
            long long o = (long long)j * M;
            pb[o] = p;
            rb[o] = r;
            CT vx = temp(3, j);
            const T ri = __ldg(&zt[ZT_RHOINV * nz + j]);
            bool zero_row = opt3d ? (j == 0 || j == nz - 1) : (j == 0);
            if (opt3d) {
                CT vy = temp(4, j);
                CT rvx = -ri * imul(kx, p);
                CT rvy = -ri * imul(ky, p);
                if (A.damp) { rvx = rvx - gd * vx; rvy = rvy - gd * vy; }
                if (zero_row) { rvx = czero<CT>(); rvy = czero<CT>(); vx = czero<CT>(); vy = czero<CT>(); }
                scr[3 * fs + o] = rvx;
                scr[4 * fs + o] = rvy;
                scr[0 * fs + o] = vx;
                scr[1 * fs + o] = vy;
            } else {
                CT rvx = -ri * imul(kx, p);
                if (zero_row) { rvx = czero<CT>(); vx = czero<CT>(); }
                scr[3 * fs + o] = rvx;
                scr[0 * fs + o] = vx;
                scr[4 * fs + o] = czero<CT>();
                scr[1 * fs + o] = czero<CT>();
            }
        }
    }

    // ---------------- S3: dp'/dz, forward elimination ------------------------
    compact_forward<CT, T>(nz, bcp, [&](int j) { return pb[(long long)j * M]; }, czero<CT>(), czero<CT>(),
                           zt + (ZT_TH + 3 * bcp) * nz, zt + (ZT_TH + 3 * bcp + 1) * nz, A.cc, y, M);

    // ---------------- S4: back substitution, RHS v_z, xi_z -------------------
    {
        const T* gam = zt + (ZT_TH + 3 * bcp + 2) * nz;
        // forcing of this step for this mode, on this slot's clock
        CT F = czero<CT>();
        const int tl = *A.clk.time - A.clk.t0[s];
        const bool src_on = A.src_mode != 0 && slot_src_on(A.clk, tl);
        if (src_on) {
            const CT* pl = A.planes + (long long)s * A.plane_ss + m;
            if (A.src_mode == 1) {
                T w = (tl < A.nseries) ? (T)A.series[(long long)s * A.nseries + tl] : (T)0;
                F = w * pl[0];
            } else {
                int idx[7];
                double w[7];
                const int nw = lagrange_dev(A.clk, tl, A.L, idx, w);
                #pragma unroll
                for (int l = 0; l < 7; ++l)
                    if (l < nw) F = F + (T)w[l] * pl[(long long)idx[l] * M];
            }
        }
        CT ud = y[(long long)(nz - 1) * M];
        for (int j = nz - 1; j >= 0; --j) {
            if (j < nz - 1) ud = y[(long long)j * M] - __ldg(&gam[j + 1]) * ud;
            CT dp = ud * __ldg(&zt[ZT_STRETCH * nz + j]);
            int ip = pmlidx(j);
            if (ip >= 0) {
                long long o = (long long)ip * M + A.ps;
                CT psi = pml[o];
                if (hs) psi = psi + beta * spml[o];
                spml[o] = __ldg(&zt[ZT_AZ * nz + j]) * dp + __ldg(&zt[ZT_BZ * nz + j]) * psi;
                dp = dp + psi;
            }
            long long o = (long long)j * M;
            CT vz = temp(5, j);
            const T ri = __ldg(&zt[ZT_RHOINV * nz + j]);
            const T gz = __ldg(&zt[ZT_G * nz + j]);
            CT r = rb[o];
            CT rv;
            if (opt3d) {
                rv = -ri * dp;
                rv = rv - (gz * ri) * r;
            } else {
                rv = -ri * (dp + gz * r);
            }
            if (src_on && j == A.ksrc) rv = rv + A.src_scale * F;
            if (A.damp) rv = rv - gd * vz;
            bool zero_row = opt3d ? (j == 0 || j == nz - 1) : (j == 0);
            if (zero_row) { rv = czero<CT>(); vz = czero<CT>(); }
            scr[5 * fs + o] = rv;
            scr[2 * fs + o] = vz;
        }
    }
}

// One RK stage of MP_QUIET_PML_3D (pml.f90:12-76), the velocity form with
// fields rho, v_x, v_y, v_z, p (initialize.f90:498-508).  Its two z
// derivatives are independent of each other:
//   S1 (up)   compact RHS of d(v_z)/dz (bc 1), forward elimination -> y
//   S2 (down) back substitution, stretch, PML psi_vz, div; the RHS of rho and
//             p are staged in rb / pb, because rho and p are still read as
//             stage arguments below
//   S3 (up)   compact RHS of dp/dz (bc 0), forward elimination -> y
//   S4 (down) back substitution, stretch, PML psi_p; RHS v_x, v_y, v_z (with
//             rho g, and the source forcing*source_dep over |k - e_rad| <= 4),
//             the staged RHS; rows 1 and nz zeroed; then the damping of v,
//             which the reference applies after the zeroing (pml.f90:57-72)
template <typename T>
__global__ void __launch_bounds__(128) stage_velocity_kernel(const StageArgs<T> A) {
    typedef typename CplxOf<T>::type CT;
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= A.M) return;
    const int s = blockIdx.y;
    const int nz = A.nz;
    const long long M = A.M, fs = A.fs;
    CT* __restrict__ a = A.a + (long long)s * 6 * fs + m;
    CT* __restrict__ scr = A.scr + (long long)s * 6 * fs + m;
    CT* __restrict__ pml = A.pml + (long long)s * 2 * A.ps + m;
    CT* __restrict__ spml = A.scrpml + (long long)s * 2 * A.ps + m;
    CT* __restrict__ y = A.ybuf + (long long)s * fs + m;
    CT* __restrict__ pb = A.pbuf + (long long)s * fs + m;
    CT* __restrict__ rb = A.rbuf + (long long)s * fs + m;
    const T* __restrict__ zt = A.zt;
    const T kx = __ldg(&A.pt[PT_KX * M + m]);
    const T ky = __ldg(&A.pt[PT_KY * M + m]);
    const T gd = A.damp ? __ldg(&A.pt[PT_DAMP * M + m]) : (T)0;
    const T beta = A.beta;
    const bool hs = A.has_scr != 0;
    const int nb = A.npmlbot, nt = A.npmltop;
    auto temp = [&](int f, int j) -> CT {
        long long o = f * fs + (long long)j * M;
        CT v = a[o];
        if (hs) v = v + beta * scr[o];
        return v;
    };
    auto pmlidx = [&](int j) -> int { return j < nb ? j : (j >= nz - nt ? nb + (j - (nz - nt)) : -1); };

    // S1: d(v_z)/dz, bc 1
    compact_forward<CT, T>(nz, 1, [&](int j) { return temp(3, j); }, czero<CT>(), czero<CT>(),
                           zt + (ZT_TH + 3) * nz, zt + (ZT_TH + 4) * nz, A.cc, y, M);
    // S2: div, staged RHS of rho (RHScont) and p (RHSp)
    {
        const T* gam = zt + (ZT_TH + 5) * nz;
        CT ud = y[(long long)(nz - 1) * M];
        for (int j = nz - 1; j >= 0; --j) {
            if (j < nz - 1) ud = y[(long long)j * M] - __ldg(&gam[j + 1]) * ud;
            CT dz = ud * __ldg(&zt[ZT_STRETCH * nz + j]);
            const int ip = pmlidx(j);
            if (ip >= 0) {
                long long o = (long long)ip * M;
                CT psi = pml[o];
                if (hs) psi = psi + beta * spml[o];
                spml[o] = __ldg(&zt[ZT_AZ * nz + j]) * dz + __ldg(&zt[ZT_BZ * nz + j]) * psi;
                dz = dz + psi;
            }
            const CT vz = temp(3, j);
            const CT div = imul(kx, temp(1, j)) + imul(ky, temp(2, j)) + dz;
            const long long o = (long long)j * M;
            rb[o] = -__ldg(&zt[ZT_GRADRHO0 * nz + j]) * vz - __ldg(&zt[ZT_RHO0 * nz + j]) * div;
            pb[o] = -__ldg(&zt[ZT_C2RHO0 * nz + j]) * div - vz * __ldg(&zt[ZT_GRADP0 * nz + j]);
        }
    }
    // S3: dp/dz, bc 0
    compact_forward<CT, T>(nz, 0, [&](int j) { return temp(4, j); }, czero<CT>(), czero<CT>(),
                           zt + ZT_TH * nz, zt + (ZT_TH + 1) * nz, A.cc, y, M);
    // S4
    {
        const T* gam = zt + (ZT_TH + 2) * nz;
        CT F = czero<CT>();
        const int tl = *A.clk.time - A.clk.t0[s];
        const bool src_on = A.src_mode != 0 && slot_src_on(A.clk, tl);
        if (src_on) {
            const CT* pl = A.planes + (long long)s * A.plane_ss + m;
            if (A.src_mode == 1) {
                T w = (tl < A.nseries) ? (T)A.series[(long long)s * A.nseries + tl] : (T)0;
                F = w * pl[0];
            } else {
                int idx[7];
                double w[7];
                const int nw = lagrange_dev(A.clk, tl, A.L, idx, w);
                #pragma unroll
                for (int l = 0; l < 7; ++l)
                    if (l < nw) F = F + (T)w[l] * pl[(long long)idx[l] * M];
            }
        }
        CT ud = y[(long long)(nz - 1) * M];
        for (int j = nz - 1; j >= 0; --j) {
            if (j < nz - 1) ud = y[(long long)j * M] - __ldg(&gam[j + 1]) * ud;
            CT dp = ud * __ldg(&zt[ZT_STRETCH * nz + j]);
            const int ip = pmlidx(j);
            if (ip >= 0) {
                long long o = (long long)ip * M + A.ps;
                CT psi = pml[o];
                if (hs) psi = psi + beta * spml[o];
                spml[o] = __ldg(&zt[ZT_AZ * nz + j]) * dp + __ldg(&zt[ZT_BZ * nz + j]) * psi;
                dp = dp + psi;
            }
            const long long o = (long long)j * M;
            const CT r = temp(0, j), vx = temp(1, j), vy = temp(2, j), vz = temp(3, j), p = temp(4, j);
            const T ri = __ldg(&zt[ZT_RHOINV * nz + j]);
            const T gz = __ldg(&zt[ZT_G * nz + j]);
            CT rvx = -ri * imul(kx, p);
            CT rvy = -ri * imul(ky, p);
            CT rvz = -ri * (dp + gz * r);
            if (src_on && abs(j - A.ksrc) <= 4) rvz = rvz + __ldg(&zt[ZT_SRCDEP * nz + j]) * F;
            CT rc = rb[o], rp = pb[o];
            if (j == 0 || j == nz - 1) {
                rc = rp = rvx = rvy = rvz = czero<CT>();
            }
            if (A.damp) { rvx = rvx - gd * vx; rvy = rvy - gd * vy; rvz = rvz - gd * vz; }
            scr[0 * fs + o] = rc;
            scr[1 * fs + o] = rvx;
            scr[2 * fs + o] = rvy;
            scr[3 * fs + o] = rvz;
            scr[4 * fs + o] = rp;
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(128) update_kernel(const UpdateArgs<T> A) {
    typedef typename CplxOf<T>::type CT;
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= A.M) return;
    const int s = blockIdx.y;
    const int nz = A.nz;
    const long long M = A.M, fs = A.fs;
    CT* __restrict__ a = A.a + (long long)s * 6 * fs + m;
    const CT* __restrict__ scr = A.scr + (long long)s * 6 * fs + m;
    const T dt = A.dt;
    const T hf = __ldg(&A.pt[PT_HF * M + m]);
    const bool opt3d = (A.option != 17);
    const bool hstep = slot_hfilter(A.clk, *A.clk.time - A.clk.t0[s]);
    for (int f = 0; f < 6; ++f) {
        CT* af = a + f * fs;
        const CT* sf = scr + f * fs;
        // FILTER_VARS_3D filters fields 1..5 horizontally (physics.f90:795,813);
        // FILTER_VARS_2D filters all six (physics2d.f90:569)
        const bool hfil = hstep && (opt3d ? (f < 5) : true);
        zfilter_stream<CT, T>(
            nz, opt3d ? 0 : 1,
            [&](int j) { long long o = (long long)j * M; return af[o] + dt * sf[o]; },
            [&](int j, CT v) { af[(long long)j * M] = hfil ? hf * v : v; });
    }
    // PML auxiliaries (step.f90:116)
    CT* pml = A.pml + (long long)s * 2 * A.ps + m;
    const CT* spml = A.scrpml + (long long)s * 2 * A.ps + m;
    for (int q = 0; q < 2 * A.nzpml; ++q) {
        long long o = (long long)q * M;
        pml[o] = pml[o] + dt * spml[o];
    }
}

// d/dz (compact FD, bc) x stretch, optionally followed by FILTER_VAR_Z, on
// complex pencils (n1 of them, stride n1 between z-levels).  Used for the
// sensitivity-kernel derivatives (ddzkern, kernels.f90:609-621).
template <typename T>
__global__ void __launch_bounds__(128) zderiv_kernel(const T* __restrict__ zt, Compact<T> cc,
                                                     const typename CplxOf<T>::type* __restrict__ in,
                                                     typename CplxOf<T>::type* __restrict__ out,
                                                     long long n1, int nz, int bc, int filter,
                                                     const typename CplxOf<T>::type* __restrict__ top_plane,
                                                     long long in_ss, long long out_ss) {
    typedef typename CplxOf<T>::type CT;
    long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= n1) return;
    const CT* b = in + blockIdx.y * in_ss + m;
    CT* o = out + blockIdx.y * out_ss + m;
    CT top = top_plane ? top_plane[m] : czero<CT>();
    compact_forward<CT, T>(nz, bc, [&](int j) { return b[(long long)j * n1]; }, czero<CT>(), top,
                           zt + (ZT_TH + 3 * bc) * nz, zt + (ZT_TH + 3 * bc + 1) * nz, cc, o, n1);
    const T* gam = zt + (ZT_TH + 3 * bc + 2) * nz;
    CT ud = o[(long long)(nz - 1) * n1];
    o[(long long)(nz - 1) * n1] = ud * zt[ZT_STRETCH * nz + nz - 1];
    for (int j = nz - 2; j >= 0; --j) {
        ud = o[(long long)j * n1] - gam[j + 1] * ud;
        o[(long long)j * n1] = ud * zt[ZT_STRETCH * nz + j];
    }
    if (filter)
        zfilter_stream<CT, T>(nz, 0, [&](int j) { return o[(long long)j * n1]; },
                              [&](int j, CT v) { o[(long long)j * n1] = v; });
}

// ddz on real pencils (physical fields), FP64: the sparc_gpu_ddz primitive
__global__ void __launch_bounds__(128) zderiv_real_kernel(const double* __restrict__ zt, Compact<double> cc,
                                                          const double* __restrict__ in, double* __restrict__ out,
                                                          long long n1, int nz, int bc) {
    long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= n1) return;
    const double* b = in + m;
    double* o = out + m;
    double bot = o[0], top = o[(long long)(nz - 1) * n1];   // caller-set rows for bc 2 / 3
    compact_forward<double, double>(nz, bc, [&](int j) { return b[(long long)j * n1]; }, bot, top,
                                    zt + (ZT_TH + 3 * bc) * nz, zt + (ZT_TH + 3 * bc + 1) * nz, cc, o, n1);
    const double* gam = zt + (ZT_TH + 3 * bc + 2) * nz;
    double ud = o[(long long)(nz - 1) * n1];
    o[(long long)(nz - 1) * n1] = ud * zt[ZT_STRETCH * nz + nz - 1];
    for (int j = nz - 2; j >= 0; --j) {
        ud = o[(long long)j * n1] - gam[j + 1] * ud;
        o[(long long)j * n1] = ud * zt[ZT_STRETCH * nz + j];
    }
}

// vz of plane kplane into record tl/steps of each slot whose clock tl is on
// the output cadence (driver.f90:455-476)
template <typename T>
__global__ void record_kernel(const typename CplxOf<T>::type* __restrict__ a, typename CplxOf<T>::type* __restrict__ rec,
                              const int* __restrict__ t0, const int* __restrict__ time, int steps, int rec_max,
                              long long fs, int M, int kplane, int field) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    const int s = blockIdx.y;
    if (m >= M) return;
    const int tl = *time - t0[s];
    if (tl < 0 || tl % steps != 0) return;
    const int r = tl / steps;
    if (r >= rec_max) return;
    rec[((long long)s * rec_max + r) * M + m] = a[(long long)s * 6 * fs + field * fs + (long long)kplane * M + m];
}

template <typename T>
void launch_record(const typename CplxOf<T>::type* a, typename CplxOf<T>::type* rec, const int* t0, const int* time,
                   int steps, int rec_max, long long fs, int M, int kplane, int field, int nsrc, cudaStream_t s) {
    dim3 grid((M + 255) / 256, nsrc);
    record_kernel<T><<<grid, 256, 0, s>>>(a, rec, t0, time, steps, rec_max, fs, M, kplane, field);
}
template void launch_record<double>(const double2*, double2*, const int*, const int*, int, int, long long, int, int,
                                    int, int, cudaStream_t);
template void launch_record<float>(const float2*, float2*, const int*, const int*, int, int, long long, int, int, int,
                                   int, cudaStream_t);

// The context's time lives on the device so that a captured sequence of
// steps replays at any time: the step kernels read it, and one thread
// advances it after each step.
__global__ void set_time_kernel(int* time, int value) { *time = value; }
__global__ void tick_kernel(int* time) { *time = *time + 1; }
void launch_set_time(int* time, int value, cudaStream_t s) { set_time_kernel<<<1, 1, 0, s>>>(time, value); }
void launch_tick(int* time, cudaStream_t s) { tick_kernel<<<1, 1, 0, s>>>(time); }

template <typename T> void launch_stage(const StageArgs<T>& A, int nsrc, cudaStream_t s) {
    const int b = A.block == 32 ? 32 : A.block == 64 ? 64 : 128;
    dim3 grid((A.M + b - 1) / b, nsrc);
    if (A.option == 2) stage_velocity_kernel<T><<<grid, b, 0, s>>>(A);
    else stage_kernel<T><<<grid, b, 0, s>>>(A);
}
template <typename T> void launch_update(const UpdateArgs<T>& A, int nsrc, cudaStream_t s) {
    const int b = A.block == 32 ? 32 : A.block == 64 ? 64 : 128;
    dim3 grid((A.M + b - 1) / b, nsrc);
    update_kernel<T><<<grid, b, 0, s>>>(A);
}
template <typename T>
void launch_zderiv(const T* zt, const Compact<T>& cc, const typename CplxOf<T>::type* in,
                   typename CplxOf<T>::type* out, long long n1, int nz, int bc, int filter,
                   const typename CplxOf<T>::type* top_plane, int nsrc, long long in_ss, long long out_ss,
                   cudaStream_t s) {
    // top_plane (bc 3) is shared by the nsrc pencil sets
    zderiv_kernel<T><<<dim3((unsigned)((n1 + 127) / 128), nsrc), 128, 0, s>>>(zt, cc, in, out, n1, nz, bc, filter,
                                                                              top_plane, in_ss, out_ss);
}
void launch_zderiv_real(const double* zt, const Compact<double>& cc, const double* in, double* out,
                        long long n1, int nz, int bc, cudaStream_t s) {
    zderiv_real_kernel<<<(unsigned)((n1 + 127) / 128), 128, 0, s>>>(zt, cc, in, out, n1, nz, bc);
}

template void launch_stage<double>(const StageArgs<double>&, int, cudaStream_t);
template void launch_stage<float>(const StageArgs<float>&, int, cudaStream_t);
template void launch_update<double>(const UpdateArgs<double>&, int, cudaStream_t);
template void launch_update<float>(const UpdateArgs<float>&, int, cudaStream_t);
template void launch_zderiv<double>(const double*, const Compact<double>&, const double2*, double2*, long long, int,
                                    int, int, const double2*, int, long long, long long, cudaStream_t);
template void launch_zderiv<float>(const float*, const Compact<float>&, const float2*, float2*, long long, int, int,
                                   int, const float2*, int, long long, long long, cudaStream_t);
