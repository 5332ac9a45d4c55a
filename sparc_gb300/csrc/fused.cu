// Fused FP32 time step: the five LDDRK stages, the update, the z filter and
// the horizontal filter of one time step in a single kernel, with the state
// of each z-pencil held on chip for the whole step.
//
// Work decomposition.  A CTA owns P = 4 consecutive horizontal modes m of one
// source.  Each mode's z-pencil is split into chunks of CH = 5 levels, one
// chunk per thread (TP = 32*W threads per pencil, W = ceil(nz / 160) warps).
//   * a (6 fields) lives in shared memory as a tile [field][mode][z]; global rows
//     [field][z][m0..m0+3] are 32 B, so the tile is loaded and stored with
//     sector-efficient cooperative copies once per step;
//   * scr (the stage right-hand side, 6 fields) lives in registers of the
//     owning thread -- every use of scr is point-wise;
//   * stencil neighbours (compact-FD right-hand sides, z filter) are exchanged
//     through a per-pencil line in shared memory;
//   * the tridiagonal solves of DBYD2/MTRIDAG (dbyd2.f90:198-201,
//     mtridag.f90:94-111) are first-order linear recurrences.  Each thread
//     runs its chunk with a zero carry-in, the chunk maps u -> B + Mc*u are
//     composed by a scan across the pencil's threads (warp shuffles, then
//     warps through shared memory), and each thread adds H(j)*carry-in, where
//     H(j) and Mc are products of the constant elimination multipliers,
//     precomputed on the host in FP64.  This is the same LU elimination and
//     back substitution as the sequential form, re-associated.
// HBM traffic per step: read a, write a (+ the PML planes and source planes),
// and scr only on steps whose right-hand side is requested (outputs).
#include "internal.cuh"

namespace {

constexpr int CH = 5;    // z-levels per thread
constexpr int P = 4;     // modes per CTA

struct Aff {             // u -> B + M u   (B complex, M real)
    float2 B;
    float M;
};

// compose: first f, then g  -> g(f(u)) = gB + gM (fB + fM u)
__device__ __forceinline__ Aff compose(Aff f, Aff g) {
    Aff r;
    r.B.x = g.B.x + g.M * f.B.x;
    r.B.y = g.B.y + g.M * f.B.y;
    r.M = g.M * f.M;
    return r;
}

__device__ __forceinline__ Aff shfl_up(Aff a, int d) {
    Aff r;
    r.B.x = __shfl_up_sync(0xffffffffu, a.B.x, d);
    r.B.y = __shfl_up_sync(0xffffffffu, a.B.y, d);
    r.M = __shfl_up_sync(0xffffffffu, a.M, d);
    return r;
}
__device__ __forceinline__ Aff shfl_down(Aff a, int d) {
    Aff r;
    r.B.x = __shfl_down_sync(0xffffffffu, a.B.x, d);
    r.B.y = __shfl_down_sync(0xffffffffu, a.B.y, d);
    r.M = __shfl_down_sync(0xffffffffu, a.M, d);
    return r;
}

// Barrier over the TP threads of one pencil (named barrier pi+1; barrier 0
// stays the CTA-wide __syncthreads).
__device__ __forceinline__ void pencil_sync(int pi, int nthreads) {
    asm volatile("bar.sync %0, %1;" ::"r"(pi + 1), "r"(nthreads) : "memory");
}

// Exclusive scan of chunk maps over the TP threads of one pencil.
// forward = true: carry flows from lower to higher t; otherwise reversed.
// Returns the composed map of all chunks before this one (identity for the first).
__device__ __forceinline__ Aff pencil_scan(Aff mine, bool forward, int t, int W, Aff* wbuf /* [W] per pencil */,
                                           int pi) {
    const int lane = t & 31, warp = t >> 5;
    Aff inc = mine;
    if (forward) {
        #pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            Aff o = shfl_up(inc, d);
            if (lane >= d) inc = compose(o, inc);
        }
    } else {
        #pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            Aff o = shfl_down(inc, d);
            if (lane + d < 32) inc = compose(o, inc);
        }
    }
    // warp totals
    if ((forward && lane == 31) || (!forward && lane == 0)) wbuf[warp] = inc;
    if (W > 1) pencil_sync(pi, 32 * W);
    // carry from the other warps
    Aff carry;
    carry.B = make_float2(0.f, 0.f);
    carry.M = 1.f;
    if (forward) {
        for (int w = 0; w < warp; ++w) carry = compose(carry, wbuf[w]);
    } else {
        for (int w = W - 1; w > warp; --w) carry = compose(carry, wbuf[w]);
    }
    // exclusive within the warp
    Aff ex;
    if (forward) {
        ex = shfl_up(inc, 1);
        if (lane == 0) { ex.B = make_float2(0.f, 0.f); ex.M = 1.f; }
    } else {
        ex = shfl_down(inc, 1);
        if (lane == 31) { ex.B = make_float2(0.f, 0.f); ex.M = 1.f; }
    }
    if (W > 1) pencil_sync(pi, 32 * W);   // wbuf may be reused by the next scan
    return compose(carry, ex);
}

}  // namespace

// scan tables per boundary code b (FP32, nz entries per row):
// row 0 ibd(j) = 1/betad(j); row 1 m(j) = -low(j)/betad(j) (m(0) = 0);
// row 2 H(j) = prod_{i=j0..j} m(i) over j's chunk; row 3 g(j) = -gam(j+1) (g(nz-1) = 0);
// row 4 G(j) = prod_{i=j..j1-1} g(i) over j's chunk

// compact right-hand side R(j) of DBYD2 for boundary code bc from the
// exchange line xp (dbyd2.f90:94-173); top is the caller-set value for bc 3
__device__ __forceinline__ float2 compact_rhs(const float2* __restrict__ xp, int j, int nz, int bc, float2 top,
                                              const Compact<float> c) {
    auto B = [&](int k) { return xp[k]; };
    if (j >= 2 && j <= nz - 3) return c.C1 * (B(j + 1) - B(j - 1)) + c.C2 * (B(j + 2) - B(j - 2));
    if (j == 1) return c.Cb[0] * B(0) + c.Cb[1] * B(1) + c.Cb[2] * B(2) + c.Cb[3] * B(3) + c.Cb[4] * B(4);
    if (j == nz - 2)
        return -(c.Cb[0] * B(nz - 1) + c.Cb[1] * B(nz - 2) + c.Cb[2] * B(nz - 3) + c.Cb[3] * B(nz - 4) +
                 c.Cb[4] * B(nz - 5));
    if (j == 0) {
        if (bc == 0 || bc == 2) return make_float2(0.f, 0.f);
        float2 r0 = c.Cf[0] * B(0) + c.Cf[1] * B(1) + c.Cf[2] * B(2) + c.Cf[3] * B(3);
        float2 r1 = c.Cb[0] * B(0) + c.Cb[1] * B(1) + c.Cb[2] * B(2) + c.Cb[3] * B(3) + c.Cb[4] * B(4);
        return (c.alpha2 * r0 - c.beta1 * r1) * c.cnst;
    }
    // j == nz - 1
    if (bc == 0) return make_float2(0.f, 0.f);
    if (bc == 3) return top;
    float2 rn1 = -(c.Cf[0] * B(nz - 1) + c.Cf[1] * B(nz - 2) + c.Cf[2] * B(nz - 3) + c.Cf[3] * B(nz - 4));
    float2 rn2 = -(c.Cb[0] * B(nz - 1) + c.Cb[1] * B(nz - 2) + c.Cb[2] * B(nz - 3) + c.Cb[3] * B(nz - 4) +
                   c.Cb[4] * B(nz - 5));
    return (c.alpha2 * rn1 - c.beta1 * rn2) * c.cnst;
}

// d/dz (without stretch) of the values in the exchange line for the owned
// levels j0 .. j0+nown-1: forward elimination and back substitution as scans
// (srow: first of the five shared-memory scan rows of this boundary code)
__device__ __forceinline__ void zsolve(const float2* __restrict__ xp, const float* __restrict__ zs, int nz, int bc,
                                       int srow, float2 top, int j0, int nown, int t, int W, Aff* wb, int pi,
                                       const Compact<float> c, float2 (&out)[CH]) {
    const float* ibd = zs + (srow + 0) * nz;
    const float* mm = zs + (srow + 1) * nz;
    const float* HH = zs + (srow + 2) * nz;
    const float* gg = zs + (srow + 3) * nz;
    const float* GG = zs + (srow + 4) * nz;
    float2 u[CH];
    float2 run = make_float2(0.f, 0.f);
    #pragma unroll
    for (int q = 0; q < CH; ++q) {
        u[q] = make_float2(0.f, 0.f);
        if (q < nown) {
            const int j = j0 + q;
            float2 R = compact_rhs(xp, j, nz, bc, top, c);
            run = ibd[j] * R + mm[j] * run;
            u[q] = run;
        }
    }
    Aff mine;
    mine.B = nown > 0 ? run : make_float2(0.f, 0.f);
    mine.M = nown > 0 ? HH[j0 + nown - 1] : 1.f;
    Aff pre = pencil_scan(mine, true, t, W, wb, pi);
    const float2 uin = pre.B;      // ud(j0-1): the exclusive map applied to 0
    #pragma unroll
    for (int q = 0; q < CH; ++q)
        if (q < nown) u[q] = u[q] + HH[j0 + q] * uin;
    // back substitution x(j) = u(j) + g(j) x(j+1)
    float2 xr = make_float2(0.f, 0.f);
    #pragma unroll
    for (int q = CH - 1; q >= 0; --q) {
        out[q] = make_float2(0.f, 0.f);
        if (q < nown) {
            const int j = j0 + q;
            xr = u[q] + gg[j] * xr;
            out[q] = xr;
        }
    }
    Aff bm;
    bm.B = nown > 0 ? xr : make_float2(0.f, 0.f);
    bm.M = nown > 0 ? GG[j0] : 1.f;
    Aff post = pencil_scan(bm, false, t, W, wb, pi);
    const float2 xin = post.B;     // x(j1) from the next chunk
    #pragma unroll
    for (int q = 0; q < CH; ++q)
        if (q < nown) out[q] = out[q] + GG[j0 + q] * xin;
}

// shared-memory z tables: 9 profile rows, then the 5 scan rows of the
// xi_z boundary code, then the 5 of the p' boundary code
enum { ZS_STRETCH = 0, ZS_C2RHO0, ZS_GRADP0, ZS_RHO0, ZS_GRADRHO0, ZS_RHOINV, ZS_G, ZS_AZ, ZS_BZ,
       ZS_SX = 9, ZS_SP = 14, ZS_COUNT = 19 };

__global__ void __launch_bounds__(256, 2) fused_step_kernel(const FusedArgs A) {
    extern __shared__ __align__(16) unsigned char smraw[];
    const int nz = A.nz, W = A.W, TP = 32 * W;
    const int M = A.M;
    const long long fs = A.fs;
    float2* tile = (float2*)smraw;                       // [6][P][nz] (z contiguous: conflict-free chunk access)
    float2* xch = tile + 6 * nz * P;                     // [P][nz]
    const int nzpml_ = A.nzpml;
    float2* ptile = xch + P * nz;                        // [2][nzpml][P]
    Aff* wbuf = (Aff*)(ptile + 2 * A.nzpml * P + 2);     // [P][W]
    float* zs = (float*)(wbuf + P * A.W);                // [ZS_COUNT][nz] z tables
    double* lagw = (double*)(zs + ((ZS_COUNT * nz + 1) & ~1));   // [8] Lagrange weights of this slot
    int* lagi = (int*)(lagw + 8);                                 // [8]: idx[7], count
    float2* spt = (float2*)(lagi + 8);                    // [2][nzpml][P] PML right-hand sides
    float2* rl = spt + 2 * nzpml_ * P;                   // [P][nz] rho' line
    const int pi = threadIdx.x / TP;                     // pencil within the CTA
    const int t = threadIdx.x - pi * TP;                 // chunk index
    const int m0 = blockIdx.x * P;
    const int m = m0 + pi;
    const bool mvalid = m < M;
    const int s = blockIdx.y;
    const int j0 = t * CH;
    const int nown = max(0, min(CH, nz - j0));
    float2* xp = xch + pi * nz;
    Aff* wb = wbuf + pi * W;
    const float* zt = A.zt;
    float2* gA = A.a + (long long)s * 6 * fs;
    float2* gS = A.scr + (long long)s * 6 * fs;
    float2* gP = A.pml + (long long)s * 2 * A.ps;
    const int nthr = blockDim.x;
    const int nzpml = A.nzpml;
    // 16 B vector copies need every row start z*M + m0 to be even (M even)
    const bool vec = ((M & 1) == 0) && (m0 + P <= M);

    // ---- load the a tile and the PML tile (cooperative, 32 B rows) ----
    for (int r = threadIdx.x; r < 6 * nz; r += nthr) {
        const int f = r / nz, z = r - f * nz;
        const float2* src = gA + f * fs + (long long)z * M + m0;
        float2* dst = tile + f * P * nz + z;
        if (vec) {
            float4 v0 = *(const float4*)src, v1 = *(const float4*)(src + 2);
            dst[0] = make_float2(v0.x, v0.y);
            dst[nz] = make_float2(v0.z, v0.w);
            dst[2 * nz] = make_float2(v1.x, v1.y);
            dst[3 * nz] = make_float2(v1.z, v1.w);
        } else {
            for (int q = 0; q < P; ++q) dst[q * nz] = (m0 + q < M) ? src[q] : make_float2(0.f, 0.f);
        }
    }
    for (int r = threadIdx.x; r < 2 * nzpml; r += nthr) {
        const float2* src = gP + (long long)r * M + m0;
        for (int q = 0; q < P; ++q) ptile[r * P + q] = (m0 + q < M) ? src[q] : make_float2(0.f, 0.f);
    }
    const int tl = A.clk.time - A.clk.t0[s];            // this slot's clock
    const bool src_on = A.src_mode != 0 && slot_src_on(A.clk, tl);
    if (threadIdx.x == 0 && src_on && A.src_mode == 2) {
        int idx[7];
        double w[7];
        const int n = lagrange_dev(A.clk, tl, A.L, idx, w);
        for (int l = 0; l < 7; ++l) { lagw[l] = l < n ? w[l] : 0.0; lagi[l] = l < n ? idx[l] : 0; }
        lagi[7] = n;
    }
    {
        const bool o3 = (A.option == 4);
        const int bx = o3 ? 1 : 3, bp = o3 ? 0 : 2;
        // flattened over all rows so that the 256 threads share the work evenly
        for (int r = threadIdx.x; r < ZS_COUNT * nz; r += nthr) {
            const int row = r / nz, j = r - row * nz;
            const float* src;
            if (row < 9) {
                // ZS rows 0..8 map onto ZT_STRETCH, ZT_C2RHO0..ZT_G (consecutive), ZT_AZ, ZT_BZ
                const int zr = row == 0 ? ZT_STRETCH : (row <= 6 ? ZT_C2RHO0 + (row - 1) : ZT_AZ + (row - 7));
                src = A.zt + zr * nz;
            } else if (row < 14) {
                src = A.scan + (bx * 5 + (row - 9)) * nz;
            } else {
                src = A.scan + (bp * 5 + (row - 14)) * nz;
            }
            zs[r] = src[j];
        }
    }
    __syncthreads();

    const float kx = mvalid ? A.pt[PT_KX * M + m] : 0.f;
    const float ky = mvalid ? A.pt[PT_KY * M + m] : 0.f;
    const float gd = (mvalid && A.damp) ? A.pt[PT_DAMP * M + m] : 0.f;
    const bool opt3d = (A.option == 4);
    const int bcx = opt3d ? 1 : 3, bcp = opt3d ? 0 : 2;
    const int nb = A.npmlbot, nt = A.npmltop;
    // forcing of this step for this mode
    float2 F = make_float2(0.f, 0.f);
    if (src_on && mvalid) {
        const float2* pl = A.planes + (long long)s * A.plane_ss + m;
        if (A.src_mode == 1) {
            float w = (tl < A.nseries) ? (float)A.series[(long long)s * A.nseries + tl] : 0.f;
            F = w * pl[0];
        } else {
            const int nw = lagi[7];
            #pragma unroll
            for (int l = 0; l < 7; ++l)
                if (l < nw) F = F + (float)lagw[l] * pl[(long long)lagi[l] * M];
        }
    }

    float2 sc[6][CH];
    #pragma unroll
    for (int f = 0; f < 6; ++f)
        #pragma unroll
        for (int q = 0; q < CH; ++q) sc[f][q] = make_float2(0.f, 0.f);

    auto TA = [&](int f, int j) -> float2 { return tile[(f * P + pi) * nz + j]; };
    auto pmlidx = [&](int j) -> int { return j < nb ? j : (j >= nz - nt ? nb + (j - (nz - nt)) : -1); };


    for (int rk = 0; rk < 5; ++rk) {
        // static parameter indices keep the argument block out of local memory
        const float beta = rk == 0 ? A.betas[0] : rk == 1 ? A.betas[1] : rk == 2 ? A.betas[2]
                         : rk == 3 ? A.betas[3] : A.betas[4];
        const bool hs = rk > 0;
        // ---- d(xi_z)/dz ----
        #pragma unroll
        for (int q = 0; q < CH; ++q)
            if (q < nown) {
                const int j = j0 + q;
                float2 v = TA(2, j);
                if (hs) v = v + beta * sc[2][q];
                xp[j] = v;
            }
        float2 top = make_float2(0.f, 0.f);
        if (!opt3d && nown > 0 && j0 + nown == nz) {   // physics2d.f90:960
            float2 xx = TA(0, nz - 1);
            if (hs) {
                // select chain (no indexed access: sc must stay in registers)
                float2 last = sc[0][0];
                if (nown > 1) last = sc[0][1];
                if (nown > 2) last = sc[0][2];
                if (nown > 3) last = sc[0][3];
                if (nown > 4) last = sc[0][4];
                xx = xx + beta * last;
            }
            top = -(imul(kx, xx) * zt[ZT_UNSTRETCH * nz + nz - 1]);
        }
        pencil_sync(pi, TP);
        float2 dz[CH];
        zsolve(xp, zs, nz, bcx, ZS_SX, top, j0, nown, t, W, wb, pi, A.cc, dz);
        // ---- div, p', rho', horizontal right-hand sides ----
        float2 pv[CH];
        #pragma unroll
        for (int q = 0; q < CH; ++q) {
            if (q < nown) {
                const int j = j0 + q;
                float2 d = dz[q] * zs[ZS_STRETCH * nz + j];
                const int ip = pmlidx(j0 + q);
                if (ip >= 0) {
                    float2 psi = ptile[ip * P + pi];
                    if (hs) psi = psi + beta * spt[ip * P + pi];
                    spt[ip * P + pi] = zs[ZS_AZ * nz + j] * d + zs[ZS_BZ * nz + j] * psi;
                    d = d + psi;
                }
                float2 xx = TA(0, j), xy = TA(1, j), xz = TA(2, j), vx = TA(3, j), vy = TA(4, j);
                if (hs) {
                    xx = xx + beta * sc[0][q]; xy = xy + beta * sc[1][q]; xz = xz + beta * sc[2][q];
                    vx = vx + beta * sc[3][q]; vy = vy + beta * sc[4][q];
                }
                float2 div = opt3d ? imul(kx, xx) + imul(ky, xy) + d : imul(kx, xx) + d;
                float2 p = -zs[ZS_C2RHO0 * nz + j] * div - zs[ZS_GRADP0 * nz + j] * xz;
                rl[pi * nz + j] = -zs[ZS_RHO0 * nz + j] * div - zs[ZS_GRADRHO0 * nz + j] * xz;
                pv[q] = p;
                const float ri = zs[ZS_RHOINV * nz + j];
                const bool zero_row = opt3d ? (j == 0 || j == nz - 1) : (j == 0);
                if (opt3d) {
                    float2 rvx = -ri * imul(kx, p), rvy = -ri * imul(ky, p);
                    if (A.damp) { rvx = rvx - gd * vx; rvy = rvy - gd * vy; }
                    if (zero_row) { rvx = rvy = vx = vy = make_float2(0.f, 0.f); }
                    sc[3][q] = rvx; sc[4][q] = rvy; sc[0][q] = vx; sc[1][q] = vy;
                } else {
                    float2 rvx = -ri * imul(kx, p);
                    if (zero_row) { rvx = vx = make_float2(0.f, 0.f); }
                    sc[3][q] = rvx; sc[0][q] = vx;
                    sc[4][q] = make_float2(0.f, 0.f); sc[1][q] = make_float2(0.f, 0.f);
                }
            }
        }
        pencil_sync(pi, TP);   // every thread has read its xi_z neighbours
        #pragma unroll
        for (int q = 0; q < CH; ++q)
            if (q < nown) xp[j0 + q] = pv[q];
        pencil_sync(pi, TP);
        // ---- dp'/dz, RHS v_z and xi_z ----
        float2 dp[CH];
        zsolve(xp, zs, nz, bcp, ZS_SP, make_float2(0.f, 0.f), j0, nown, t, W, wb, pi, A.cc, dp);
        #pragma unroll
        for (int q = 0; q < CH; ++q) {
            if (q < nown) {
                const int j = j0 + q;
                float2 d = dp[q] * zs[ZS_STRETCH * nz + j];
                const int ip = pmlidx(j0 + q);
                if (ip >= 0) {
                    float2 psi = ptile[(nzpml + ip) * P + pi];
                    if (hs) psi = psi + beta * spt[(nzpml + ip) * P + pi];
                    spt[(nzpml + ip) * P + pi] = zs[ZS_AZ * nz + j] * d + zs[ZS_BZ * nz + j] * psi;
                    d = d + psi;
                }
                float2 vz = TA(5, j);
                if (hs) vz = vz + beta * sc[5][q];
                const float ri = zs[ZS_RHOINV * nz + j], gz = zs[ZS_G * nz + j];
                float2 rv;
                const float2 rh = rl[pi * nz + j];
                if (opt3d) { rv = -ri * d; rv = rv - (gz * ri) * rh; }
                else rv = -ri * (d + gz * rh);
                if (src_on && j == A.ksrc) rv = rv + A.src_scale * F;
                if (A.damp) rv = rv - gd * vz;
                const bool zero_row = opt3d ? (j == 0 || j == nz - 1) : (j == 0);
                if (zero_row) { rv = make_float2(0.f, 0.f); vz = make_float2(0.f, 0.f); }
                sc[5][q] = rv;
                sc[2][q] = vz;
            }
        }
        pencil_sync(pi, TP);   // exchange line free for the next stage
    }

    // ---- update a += dt*scr, pml += dt*scrpml (step.f90:114-116) ----
    const float dt = A.dt;
    #pragma unroll
    for (int f = 0; f < 6; ++f)
        #pragma unroll
        for (int q = 0; q < CH; ++q)
            if (q < nown) {
                const int j = j0 + q;
                tile[(f * P + pi) * nz + j] = tile[(f * P + pi) * nz + j] + dt * sc[f][q];
            }
    #pragma unroll
    for (int q = 0; q < CH; ++q)
        if (q < nown) {
            const int ip = pmlidx(j0 + q);
            if (ip >= 0) {
                ptile[ip * P + pi] = ptile[ip * P + pi] + dt * spt[ip * P + pi];
                ptile[(nzpml + ip) * P + pi] = ptile[(nzpml + ip) * P + pi] + dt * spt[(nzpml + ip) * P + pi];
            }
        }
    pencil_sync(pi, TP);
    // ---- z filter (+ horizontal filter) into registers, then back into the tile ----
    const float hf = mvalid ? A.pt[PT_HF * M + m] : 1.f;
    const float h1 = 0.5f * 0.41015625f, h2 = 0.5f * -0.234375f, h3 = 0.5f * 0.087890625f;
    const float h4 = 0.5f * -0.01953125f, h5 = 0.5f * 0.001953125f, c0 = 0.75390625f;
    #pragma unroll
    for (int f = 0; f < 6; ++f) {
        const bool hfil = slot_hfilter(A.clk, tl) && (opt3d ? (f < 5) : true);
        float2 out[CH];
        #pragma unroll
        for (int q = 0; q < CH; ++q) {
            if (q < nown) {
                const int j = j0 + q;
                auto V = [&](int k) { return tile[(f * P + pi) * nz + k]; };
                float2 o;
                const bool near_bot = (j >= 1 && j <= 4), near_top = (j >= nz - 5 && j <= nz - 2);
                if (j == 0 || j == nz - 1) o = V(j);
                else if (near_top) o = 0.5f * (V(j + 1) + V(j - 1));
                else if (near_bot) o = opt3d ? 0.5f * (V(j + 1) + V(j - 1)) : V(j);
                else
                    o = c0 * V(j) + h1 * (V(j - 1) + V(j + 1)) + h2 * (V(j - 2) + V(j + 2)) +
                        h3 * (V(j - 3) + V(j + 3)) + h4 * (V(j - 4) + V(j + 4)) + h5 * (V(j - 5) + V(j + 5));
                out[q] = hfil ? hf * o : o;
            }
        }
        pencil_sync(pi, TP);
        #pragma unroll
        for (int q = 0; q < CH; ++q)
            if (q < nown) tile[(f * P + pi) * nz + j0 + q] = out[q];
    }
    __syncthreads();   // the store below copies every pencil's rows
    // ---- store a and the PML planes ----
    for (int r = threadIdx.x; r < 6 * nz; r += nthr) {
        const int f = r / nz, z = r - f * nz;
        float2* dst = gA + f * fs + (long long)z * M + m0;
        const float2* srcp = tile + f * P * nz + z;
        if (vec) {
            float2 w0 = srcp[0], w1 = srcp[nz], w2 = srcp[2 * nz], w3 = srcp[3 * nz];
            *(float4*)dst = make_float4(w0.x, w0.y, w1.x, w1.y);
            *(float4*)(dst + 2) = make_float4(w2.x, w2.y, w3.x, w3.y);
        } else {
            for (int q = 0; q < P; ++q)
                if (m0 + q < M) dst[q] = srcp[q * nz];
        }
    }
    for (int r = threadIdx.x; r < 2 * nzpml; r += nthr) {
        float2* dst = gP + (long long)r * M + m0;
        for (int q = 0; q < P; ++q)
            if (m0 + q < M) dst[q] = ptile[r * P + q];
    }
    // ---- the last stage's right-hand side, when an output needs it ----
    if (A.write_scr) {
        __syncthreads();
        #pragma unroll
        for (int f = 0; f < 6; ++f)
            #pragma unroll
            for (int q = 0; q < CH; ++q)
                if (q < nown) tile[(f * P + pi) * nz + j0 + q] = sc[f][q];
        __syncthreads();
        for (int f = 0; f < 6; ++f)
        for (int z = threadIdx.x; z < nz; z += nthr) {
            float2* dst = gS + f * fs + (long long)z * M + m0;
            const float2* srcp = tile + f * P * nz + z;
            if (vec) {
                float2 w0 = srcp[0], w1 = srcp[nz], w2 = srcp[2 * nz], w3 = srcp[3 * nz];
                *(float4*)dst = make_float4(w0.x, w0.y, w1.x, w1.y);
                *(float4*)(dst + 2) = make_float4(w2.x, w2.y, w3.x, w3.y);
            } else {
                for (int q = 0; q < P; ++q)
                    if (m0 + q < M) dst[q] = srcp[q * nz];
            }
        }
    }
}

size_t fused_smem_bytes(int nz, int nzpml, int W) {
    return (size_t)(6 * nz * P + P * nz + 2 * nzpml * P + 2) * sizeof(float2) + (size_t)P * W * sizeof(Aff) +
           (size_t)(ZS_COUNT * nz + 2) * sizeof(float) + 8 * sizeof(double) + 8 * sizeof(int) +
           (size_t)(2 + 2 * nzpml * P + P * nz) * sizeof(float2) + 16;
}

int fused_supported(int nz) { return nz <= 2 * 32 * CH; }

void launch_fused(const FusedArgs& A, int nsrc, cudaStream_t s) {
    const int TP = 32 * A.W;
    const size_t sm = fused_smem_bytes(A.nz, A.nzpml, A.W);
    cudaFuncSetAttribute((const void*)fused_step_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    dim3 grid((A.M + P - 1) / P, nsrc);
    fused_step_kernel<<<grid, P * TP, sm, s>>>(A);
}
