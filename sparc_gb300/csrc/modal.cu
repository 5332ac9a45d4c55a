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

// ---------------------------------------------------------------------------
// The same RK stage with each z-pencil cut into Q chunks of C levels, one
// chunk per lane (the Q lanes of a mode are consecutive lanes of one warp).
// A pencil's two tridiagonal solves are first-order recurrences: each lane
// eliminates its chunk with a zero carry, the chunk maps u -> B + M u are
// composed by a scan over the Q lanes (warp shuffles, exact FP64 products),
// and each level adds H(j) times the carry, H(j) the product of the
// multipliers from the chunk start to j (host FP64, table zc); the back
// substitution likewise from above with G(j).  This is the elimination and
// back substitution of the one-lane form (mtridag.f90:94-111), re-associated.
// Per solve three passes over the chunk: up (right-hand side, zero-carry
// elimination -> y), down (fix with H, zero-carry back substitution -> y),
// and the fix with G feeding the point-wise work of the one-lane form's S2 /
// S4.  The p' neighbours of the second solve come from the other lanes'
// chunks in global memory, after a warp barrier.  Q > 1 puts Q times more
// warps on small grids (8320 modes at 128x128), which the FP64 pipe needs.
// ---------------------------------------------------------------------------
template <typename T> struct AffZ {
    typename CplxOf<T>::type B;
    T M;
};

template <typename T, int Q, bool FWD>
__device__ __forceinline__ typename CplxOf<T>::type chunk_scan(typename CplxOf<T>::type B, T M, int c) {
    typedef typename CplxOf<T>::type CT;
    // inclusive scan over the Q lanes of a mode (FWD: from chunk 0 up; else
    // from chunk Q-1 down), then the exclusive carry into this chunk
    CT b = B;
    T mm = M;
    #pragma unroll
    for (int d = 1; d < Q; d <<= 1) {
        CT ob;
        T om;
        if (FWD) {
            ob.x = __shfl_up_sync(0xffffffffu, b.x, d, Q); ob.y = __shfl_up_sync(0xffffffffu, b.y, d, Q);
            om = __shfl_up_sync(0xffffffffu, mm, d, Q);
        } else {
            ob.x = __shfl_down_sync(0xffffffffu, b.x, d, Q); ob.y = __shfl_down_sync(0xffffffffu, b.y, d, Q);
            om = __shfl_down_sync(0xffffffffu, mm, d, Q);
        }
        if (FWD ? (c >= d) : (c + d < Q)) {      // this chunk's map after the other's
            b = b + mm * ob;
            mm = mm * om;
        }
    }
    CT ex;
    if (FWD) {
        ex.x = __shfl_up_sync(0xffffffffu, b.x, 1, Q); ex.y = __shfl_up_sync(0xffffffffu, b.y, 1, Q);
        if (c == 0) ex = czero<CT>();
    } else {
        ex.x = __shfl_down_sync(0xffffffffu, b.x, 1, Q); ex.y = __shfl_down_sync(0xffffffffu, b.y, 1, Q);
        if (c == Q - 1) ex = czero<CT>();
    }
    return ex;
}

// Right-hand side of the compact first derivative at level j (dbyd2.f90:
// 88-173) of the values ld(j'), boundary code bc; bot / top: the caller-set
// values of bc 2 / 3.
template <typename CT, typename T, typename Load>
__device__ __forceinline__ CT compact_rhs(int j, int nz, int bc, Load ld, CT bot, CT top, const Compact<T>& c) {
    if (j >= 2 && j <= nz - 3) return c.C1 * (ld(j + 1) - ld(j - 1)) + c.C2 * (ld(j + 2) - ld(j - 2));
    if (j <= 1) {
        const CT b0 = ld(0), b1 = ld(1), b2 = ld(2), b3 = ld(3), b4 = ld(4);
        const CT r1 = c.Cb[0] * b0 + c.Cb[1] * b1 + c.Cb[2] * b2 + c.Cb[3] * b3 + c.Cb[4] * b4;
        if (j == 1) return r1;
        if (bc == 0) return czero<CT>();
        if (bc == 2) return bot;
        const CT r0 = c.Cf[0] * b0 + c.Cf[1] * b1 + c.Cf[2] * b2 + c.Cf[3] * b3;
        return (c.alpha2 * r0 - c.beta1 * r1) * c.cnst;
    }
    const CT b0 = ld(nz - 1), b1 = ld(nz - 2), b2 = ld(nz - 3), b3 = ld(nz - 4), b4 = ld(nz - 5);
    const CT rn2 = -(c.Cb[0] * b0 + c.Cb[1] * b1 + c.Cb[2] * b2 + c.Cb[3] * b3 + c.Cb[4] * b4);
    if (j == nz - 2) return rn2;
    if (bc == 0) return czero<CT>();
    if (bc == 3) return top;
    const CT rn1 = -(c.Cf[0] * b0 + c.Cf[1] * b1 + c.Cf[2] * b2 + c.Cf[3] * b3);
    return (c.alpha2 * rn1 - c.beta1 * rn2) * c.cnst;
}

// One chunked solve: d/dz (without stretch) of ld over the lane's chunk
// [j0, j1) of boundary code bc; y: the pencil's scratch column (this lane's
// levels only; written only when store, i.e. by lanes of real modes).
// emit(j, dz) is called for every level of the chunk, top down.  zh, zg: the
// H and G rows of bc for this chunking.
template <typename T, int Q, typename Load, typename Emit>
__device__ __forceinline__ void chunk_solve(int j0, int j1, int c, int nz, int bc, Load ld,
                                            typename CplxOf<T>::type top, const T* __restrict__ low,
                                            const T* __restrict__ ibd, const T* __restrict__ gam,
                                            const T* __restrict__ zh, const T* __restrict__ zg, const Compact<T>& cc,
                                            typename CplxOf<T>::type* __restrict__ y, long long M, bool store,
                                            Emit emit) {
    typedef typename CplxOf<T>::type CT;
    // up: zero-carry elimination UD(J) = (R(J) - A(J) UD(J-1)) / BETAD(J)
    CT run = czero<CT>();
    for (int j = j0; j < j1; ++j) {
        const CT R = compact_rhs<CT, T>(j, nz, bc, ld, czero<CT>(), top, cc);
        run = (R - __ldg(&low[j]) * run) * __ldg(&ibd[j]);
        if (store) y[(long long)j * M] = run;
    }
    const CT uin = chunk_scan<T, Q, true>(run, j1 > j0 ? __ldg(&zh[j1 - 1]) : (T)1, c);
    // down: UD(J) = y(J) + H(J) uin, then zero-carry back substitution
    CT x = czero<CT>();
    for (int j = j1 - 1; j >= j0; --j) {
        const CT ud = y[(long long)j * M] + __ldg(&zh[j]) * uin;
        x = (j == j1 - 1) ? ud : ud - __ldg(&gam[j + 1]) * x;
        if (store) y[(long long)j * M] = x;
    }
    const CT xin = chunk_scan<T, Q, false>(x, j1 > j0 ? __ldg(&zg[j0]) : (T)1, c);
    for (int j = j1 - 1; j >= j0; --j) emit(j, y[(long long)j * M] + __ldg(&zg[j]) * xin);
}

template <typename T, int Q>
__global__ void __launch_bounds__(128) stage_chunk_kernel(const StageArgs<T> A) {
    typedef typename CplxOf<T>::type CT;
    const int gt = blockIdx.x * blockDim.x + threadIdx.x;
    const int c = gt % Q;
    const int m0 = gt / Q;
    const bool valid = m0 < A.M;
    const int m = valid ? m0 : A.M - 1;      // lanes past the last mode repeat it and store nothing
    const int s = blockIdx.y;
    const int nz = A.nz, C = A.chunk;
    const int j0 = c * C, j1 = min(j0 + C, nz);
    const long long M = A.M, fs = A.fs;
    CT* __restrict__ a = A.a + (long long)s * 6 * fs + m;
    CT* __restrict__ scr = A.scr + (long long)s * 6 * fs + m;
    CT* __restrict__ pml = A.pml + (long long)s * 2 * A.ps + m;
    CT* __restrict__ spml = A.scrpml + (long long)s * 2 * A.ps + m;
    CT* __restrict__ y = A.ybuf + (long long)s * fs + m;
    CT* __restrict__ pb = A.pbuf + (long long)s * fs + m;
    CT* __restrict__ rb = A.rbuf + (long long)s * fs + m;
    const T* __restrict__ zt = A.zt;
    const T* __restrict__ zc = A.zc;
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

    // ---- solve 1: d(xi_z)/dz; then div, p', rho' and the horizontal RHS (S2) ----
    CT top = czero<CT>();
    if (!opt3d && j1 == nz) {   // physics2d.f90:960: dxizdz(nz) = -dxixdx(nz) * unstretch(nz)
        CT xx = temp(0, nz - 1);
        top = -(imul(kx, xx) * __ldg(&zt[ZT_UNSTRETCH * nz + nz - 1]));
    }
    chunk_solve<T, Q>(j0, j1, c, nz, bcx, [&](int j) { return temp(2, j); }, top, zt + (ZT_TH + 3 * bcx) * nz,
                      zt + (ZT_TH + 3 * bcx + 1) * nz, zt + (ZT_TH + 3 * bcx + 2) * nz, zc, zc + nz, A.cc, y, M,
                      valid, [&](int j, CT ud) {
        if (!valid) return;
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
    });
    // the second solve reads p' two levels into the neighbouring chunks
    __syncwarp();

    // ---- solve 2: dp'/dz; RHS v_z (+ source, damping) and xi_z (S4) ----
    CT F = czero<CT>();
    const int tl = *A.clk.time - A.clk.t0[s];
    const bool src_on = A.src_mode != 0 && slot_src_on(A.clk, tl) && A.ksrc >= j0 && A.ksrc < j1;
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
    chunk_solve<T, Q>(j0, j1, c, nz, bcp, [&](int j) { return pb[(long long)j * M]; }, czero<CT>(),
                      zt + (ZT_TH + 3 * bcp) * nz, zt + (ZT_TH + 3 * bcp + 1) * nz, zt + (ZT_TH + 3 * bcp + 2) * nz,
                      zc + 2 * nz, zc + 3 * nz, A.cc, y, M, valid, [&](int j, CT ud) {
        if (!valid) return;
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
    });
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

// z filter of FILTER_VARS_3D / _2D (physics.f90:758-786, physics2d.f90:531-561)
// at one level j of a pencil whose values ld(j') are all available; the same
// formulas, in the same order, as zfilter_stream.
template <typename V, typename T, typename Load>
__device__ __forceinline__ V zfilter_at(int j, int nz, int mode, Load ld) {
    const T h1 = (T)(0.5 * 0.41015625), h2 = (T)(0.5 * -0.234375), h3 = (T)(0.5 * 0.087890625);
    const T h4 = (T)(0.5 * -0.01953125), h5 = (T)(0.5 * 0.001953125), c0 = (T)0.75390625, hf = (T)0.5;
    if (j == 0 || j == nz - 1) return ld(j);
    if (j >= nz - 5 && j <= nz - 2) return hf * (ld(j + 1) + ld(j - 1));
    if (j >= 1 && j <= 4) return (mode == 0) ? hf * (ld(j + 1) + ld(j - 1)) : ld(j);
    return c0 * ld(j) + h1 * (ld(j - 1) + ld(j + 1)) + h2 * (ld(j - 2) + ld(j + 2)) +
           h3 * (ld(j - 3) + ld(j + 3)) + h4 * (ld(j - 4) + ld(j + 4)) + h5 * (ld(j - 5) + ld(j + 5));
}

// update_kernel with each pencil on Q lanes of a warp (chunks of A.chunk
// levels): per field, a + dt*scr of the lane's chunk goes to the pencil's
// scratch column y, and after a warp barrier the z filter reads its
// neighbours there and writes a.  Arithmetic identical to update_kernel.
template <typename T, int Q>
__global__ void __launch_bounds__(128) update_chunk_kernel(const UpdateArgs<T> A) {
    typedef typename CplxOf<T>::type CT;
    const int gt = blockIdx.x * blockDim.x + threadIdx.x;
    const int c = gt % Q;
    const int m0 = gt / Q;
    const bool valid = m0 < A.M;
    const int m = valid ? m0 : A.M - 1;
    const int s = blockIdx.y;
    const int nz = A.nz, C = A.chunk;
    const int j0 = c * C, j1 = min(j0 + C, nz);
    const long long M = A.M, fs = A.fs;
    CT* __restrict__ a = A.a + (long long)s * 6 * fs + m;
    const CT* __restrict__ scr = A.scr + (long long)s * 6 * fs + m;
    CT* __restrict__ y = A.ybuf + (long long)s * fs + m;
    const T dt = A.dt;
    const T hf = __ldg(&A.pt[PT_HF * M + m]);
    const bool opt3d = (A.option != 17);
    const bool hstep = slot_hfilter(A.clk, *A.clk.time - A.clk.t0[s]);
    for (int f = 0; f < 6; ++f) {
        CT* af = a + f * fs;
        const CT* sf = scr + f * fs;
        const bool hfil = hstep && (opt3d ? (f < 5) : true);
        if (valid)
            for (int j = j0; j < j1; ++j) {
                const long long o = (long long)j * M;
                y[o] = af[o] + dt * sf[o];
            }
        __syncwarp();
        if (valid)
            for (int j = j0; j < j1; ++j) {
                const CT v = zfilter_at<CT, T>(j, nz, opt3d ? 0 : 1, [&](int jj) { return y[(long long)jj * M]; });
                af[(long long)j * M] = hfil ? hf * v : v;
            }
        __syncwarp();      // the next field overwrites y
    }
    if (valid) {
        CT* pml = A.pml + (long long)s * 2 * A.ps + m;
        const CT* spml = A.scrpml + (long long)s * 2 * A.ps + m;
        for (int q = c; q < 2 * A.nzpml; q += Q) {
            const long long o = (long long)q * M;
            pml[o] = pml[o] + dt * spml[o];
        }
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
    if (A.option != 2 && A.q > 1) {
        dim3 grid((unsigned)(((long long)A.M * A.q + b - 1) / b), nsrc);
        if (A.q == 2) stage_chunk_kernel<T, 2><<<grid, b, 0, s>>>(A);
        else if (A.q == 4) stage_chunk_kernel<T, 4><<<grid, b, 0, s>>>(A);
        else stage_chunk_kernel<T, 8><<<grid, b, 0, s>>>(A);
        return;
    }
    dim3 grid((A.M + b - 1) / b, nsrc);
    if (A.option == 2) stage_velocity_kernel<T><<<grid, b, 0, s>>>(A);
    else stage_kernel<T><<<grid, b, 0, s>>>(A);
}
template <typename T> void launch_update(const UpdateArgs<T>& A, int nsrc, cudaStream_t s) {
    const int b = A.block == 32 ? 32 : A.block == 64 ? 64 : 128;
    if (A.q > 1) {
        dim3 grid((unsigned)(((long long)A.M * A.q + b - 1) / b), nsrc);
        if (A.q == 2) update_chunk_kernel<T, 2><<<grid, b, 0, s>>>(A);
        else if (A.q == 4) update_chunk_kernel<T, 4><<<grid, b, 0, s>>>(A);
        else update_chunk_kernel<T, 8><<<grid, b, 0, s>>>(A);
        return;
    }
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
