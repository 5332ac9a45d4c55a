// Fused FP32 time step: the five LDDRK stages, the update, the z filter and
// the horizontal filter of one time step in a single kernel, with the state
// of each z-pencil held on chip for the whole step.
//
// Work decomposition.  A work item is P = 2, 4 or 8 consecutive horizontal
// modes m of one source; the launch has one CTA per resident slot (one per SM
// at P = 8), and CTA b takes items b, b + G, b + 2G, ... (G CTAs), loading the
// z tables once and issuing each item's tile copies right after the previous
// item's stores have read the tile out of shared memory.  Each mode's
// z-pencil is split into chunks of CH = 5 levels, one chunk per thread:
// TP = 32*W threads per pencil, W = ceil(nz / 160) warps, and the pencil is
// padded to NZP = TP*CH levels.
//   * a (6 fields) lives in shared memory as a tile [field][mode][z] with
//     zero ghost rows on both ends; global rows [field][z][m0..m0+P-1] are
//     8P bytes, so the tile is loaded (cp.async, each value into its
//     transposed place) and stored (P/2 lanes per row, one float4 each, so
//     a warp store covers whole rows) with sector-efficient cooperative
//     copies once per step;
//   * scr (the stage right-hand side, 6 fields) lives in registers of the
//     owning thread -- every use of scr is point-wise;
//   * stencil neighbours of the compact-FD right-hand sides are exchanged
//     through two per-pencil lines in shared memory (xi_z, then p'), so a
//     stage needs one barrier per line;
//   * every thread evaluates the interior formulas (compact right-hand side,
//     11-point z filter) on all of its levels -- the ghost and padding rows
//     make that safe -- and the few threads that own boundary rows, PML
//     planes or the source plane then overwrite those rows.  The main path is
//     the same instruction stream for every thread of a warp;
//   * the tridiagonal solves of DBYD2/MTRIDAG (dbyd2.f90:198-201,
//     mtridag.f90:94-111) are first-order linear recurrences.  Each thread
//     runs its chunk with a zero carry-in; the chunk maps u -> B + Mc*u then
//     give the carry into chunk t as the sum over the preceding chunks of
//     B(t-i) times the product of the multipliers Mc between them (and the
//     same from above for the back substitution).  Those products depend on
//     z only (the matrix is the same for every mode), shrink by about 0.008
//     per chunk (|multiplier| ~ 0.38 per level), and are precomputed on the
//     host in FP64: the sum is taken over the KB = 5 nearest chunks, read
//     from a per-pencil line in shared memory after one barrier.  The terms
//     left out are below 2^-32 of a chunk value (checked on the host for
//     every boundary code, else the context runs the per-stage kernels).
//     Each thread back-substitutes its chunk with zero carries before the
//     first barrier, and the carries enter afterwards as
//     x(j) = x0(j) + K(j)*carry-in + G(j)*carry-from-above, K and G host
//     tables (K(j) = H(j) + g(j) K(j+1), H(j) the product of the multipliers
//     from the chunk start to j).  This is the LU elimination and back
//     substitution of the sequential form, re-associated.  Padding
//     rows carry zero multipliers, so they never reach a real row.  The
//     tables solve for the scaled unknown s(j) x(j) (s = stretch for xi_z,
//     stretch / rho0 for p'), so each solve returns the derivative in the
//     form the step uses, without a multiply and a table read per level;
//   * the state tile of the CTA that starts one resident-CTA count later is
//     prefetched into L2 while this CTA computes, so its load phase reads L2;
//   * a LAGRANGE_INTERP source (the adjoint's) is interpolated to the step by
//     a small kernel launched before it (source_plane_kernel), so no CTA
//     spends its critical path on the seven FP64 weights.
// HBM traffic per step: read a, write a (+ the PML planes and source planes),
// and scr only on steps whose right-hand side is requested (outputs).
#include <algorithm>
#include <type_traits>

#include "internal.cuh"

namespace {

constexpr int CH = FUSED_CH;   // z-levels per thread
constexpr int GZ = 5;          // ghost rows of the tile on each side (reach of the z filter)
constexpr int GX = 2;          // ghost entries of an exchange line on each side (compact stencil)
constexpr int KB = FUSED_KB;   // chunks summed by a look-back carry

// Entry idx of the z tables (scalars in shared memory) as a pair (t, t), the
// multiplier of a paired product with a complex value.  Tables stored as
// pairs would save the broadcast but cost 24 KB of shared memory (and of L1)
// per CTA; measured slower.
__device__ __forceinline__ float2 zt2(const float* zs, int idx) {
    const float t = zs[idx];
    return make_float2(t, t);
}

// Barrier over the TP threads of one pencil (named barrier pi+1; barrier 0
// stays the CTA-wide __syncthreads).
__device__ __forceinline__ void pencil_sync(int pi, int nthreads) {
    asm volatile("bar.sync %0, %1;" ::"r"(pi + 1), "r"(nthreads) : "memory");
}

// Carry of a chunk from the KB = 5 nearest chunk values of a look-back line:
// sum over i = 1..5 of prod(i) * v(i), prod(1) = 1, prod(2..5) = pr.x..pr.w,
// as two independent partial sums (a shorter dependency chain).
__device__ __forceinline__ float2 lookback(float4 pr, float2 v1, float2 v2, float2 v3, float2 v4, float2 v5) {
    float2 c1 = pmul(bc2(pr.w), v5);
    c1 = pfma(bc2(pr.z), v4, c1);
    float2 c2 = pmul(bc2(pr.y), v3);
    c2 = pfma(bc2(pr.x), v2, c2);
    return padd(v1, padd(c1, c2));
}

// d/dz (without stretch) of the values of one exchange line (xp[j], j in
// 0..NZP-1, ghosts at -2, -1, NZP, NZP+1; own[q] = xp[j0+q]) for the owned
// levels j0..j0+CH-1,
// boundary code BC (dbyd2.f90:94-173 for the right-hand side; top is the
// caller-set value of bc 3).  zs, r0: the z tables and the first of the five
// elimination rows (1/betad, m, K, g, G) of BC; lb, lb+1: its forward and
// backward look-back product tables ([t][4] floats each); lf, lk:
// this pencil's forward and backward look-back lines (chunk t at index t,
// zero entries at -KB..-1 and TP..TP+KB-1).
template <int BC, int W>
__device__ __forceinline__ void zsolve(const float2* __restrict__ xp, const float2 (&own)[CH],
                                       const float* __restrict__ zs, int r0, int lb, int nz, float2 top, int j0,
                                       bool lo, bool hi, int t, float2* lf, float2* lk, int pi,
                                       const Compact<float> c, float2 (&out)[CH]) {
    constexpr int NZP = 160 * W;
    const int ibd = r0 * NZP, mm = (r0 + 1) * NZP, HH = (r0 + 2) * NZP, gg = (r0 + 3) * NZP, GG = (r0 + 4) * NZP;
    auto Z = [&](int row, int j) { return zt2(zs, row + j); };
    float2 u[CH];
    const float2 C1p = bc2(c.C1), C2p = bc2(c.C2);
    // interior right-hand side on every level (dbyd2.f90:88-92); the
    // thread's own levels come from registers (own[q] == xp[j0+q]), the two
    // levels on each side from the neighbours' entries of the line
    #pragma unroll
    for (int q = 0; q < CH; ++q) {
        const int j = j0 + q;
        const float2 bm2 = q >= 2 ? own[q - 2] : xp[j - 2];
        const float2 bm1 = q >= 1 ? own[q - 1] : xp[j - 1];
        const float2 bp1 = q + 1 < CH ? own[q + 1] : xp[j + 1];
        const float2 bp2 = q + 2 < CH ? own[q + 2] : xp[j + 2];
        u[q] = pfma(C2p, psub(bp2, bm2), pmul(C1p, psub(bp1, bm1)));
    }
    if (lo) {   // rows 0 and 1 (dbyd2.f90:104-173)
        const float2 b0 = own[0], b1 = own[1], b2 = own[2], b3 = own[3], b4 = own[4];   // j0 = 0
        const float2 r1 = c.Cb[0] * b0 + c.Cb[1] * b1 + c.Cb[2] * b2 + c.Cb[3] * b3 + c.Cb[4] * b4;
        u[1] = r1;
        if (BC == 0 || BC == 2) {
            u[0] = make_float2(0.f, 0.f);
        } else {
            const float2 r0 = c.Cf[0] * b0 + c.Cf[1] * b1 + c.Cf[2] * b2 + c.Cf[3] * b3;
            u[0] = (c.alpha2 * r0 - c.beta1 * r1) * c.cnst;
        }
    }
    if (hi) {   // rows nz-2 and nz-1
        const float2 b0 = xp[nz - 1], b1 = xp[nz - 2], b2 = xp[nz - 3], b3 = xp[nz - 4], b4 = xp[nz - 5];
        const float2 rm2 = -(c.Cb[0] * b0 + c.Cb[1] * b1 + c.Cb[2] * b2 + c.Cb[3] * b3 + c.Cb[4] * b4);
        float2 rm1;
        if (BC == 0) {
            rm1 = make_float2(0.f, 0.f);
        } else if (BC == 3) {
            rm1 = top;
        } else {
            const float2 rn1 = -(c.Cf[0] * b0 + c.Cf[1] * b1 + c.Cf[2] * b2 + c.Cf[3] * b3);
            rm1 = (c.alpha2 * rn1 - c.beta1 * rm2) * c.cnst;
        }
        #pragma unroll
        for (int q = 0; q < CH; ++q) {
            if (j0 + q == nz - 2) u[q] = rm2;
            if (j0 + q == nz - 1) u[q] = rm1;
        }
    }
    // forward elimination with zero carry-in, then the scan for the carry
    float2 run = make_float2(0.f, 0.f);
    #pragma unroll
    for (int q = 0; q < CH; ++q) {
        const int j = j0 + q;
        run = pfma(Z(mm, j), run, pmul(Z(ibd, j), u[q]));
        u[q] = run;
    }
    // carry into the chunk: ud(j0-1) from the chunk values below
    constexpr int TP = 32 * W;
    lf[t] = run;
    // back substitution x0(j) = u(j) + g(j) x0(j+1) with zero carries, while
    // the other chunks reach the barrier; the carries enter afterwards as
    // x(j) = x0(j) + K(j) uin + G(j) xin, K(j) = H(j) + g(j) K(j+1) (host table)
    float2 xr = make_float2(0.f, 0.f);
    #pragma unroll
    for (int q = CH - 1; q >= 0; --q) {
        xr = pfma(Z(gg, j0 + q), xr, u[q]);
        out[q] = xr;
    }
    const float4 prf = *(const float4*)(zs + lb * NZP + 4 * t);      // read before the barrier
    pencil_sync(pi, TP);
    const float2 uin = lookback(prf, lf[t - 1], lf[t - 2], lf[t - 3], lf[t - 4], lf[t - 5]);
    // carry from above: x(j0+CH) from the chunk values above
    lk[t] = pfma(Z(HH, j0), uin, xr);
    const float4 prb = *(const float4*)(zs + (lb + 1) * NZP + 4 * t);
    pencil_sync(pi, TP);
    const float2 xin = lookback(prb, lk[t + 1], lk[t + 2], lk[t + 3], lk[t + 4], lk[t + 5]);
    #pragma unroll
    for (int q = 0; q < CH; ++q) out[q] = pfma(Z(GG, j0 + q), xin, pfma(Z(HH, j0 + q), uin, out[q]));
}

// Poll phase 0 of an mbarrier at most `limit` times; true once it completed.
__device__ __forceinline__ bool mbar_wait(unsigned mbar, int limit) {
    unsigned done = 0;
    for (int it = 0; it < limit && !done; ++it)
        asm volatile("{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\nselp.u32 %0, 1, 0, p;\n}\n"
                     : "=r"(done)
                     : "r"(mbar)
                     : "memory");
    return done != 0;
}

// shared-memory layout (byte offsets), identical on host and device
struct FusedLayout {
    int tile, xl, ptile, spt, lines, zs, mbar, total;
};
__host__ __device__ inline FusedLayout fused_layout(int P, int W, int nzpml) {
    const int NZP = 160 * W, LZ = NZP + 2 * GZ, LX = NZP + 2 * GX, LL = 32 * W + 2 * KB;
    FusedLayout L;
    int o = 0;
    L.tile = o;  o += 6 * P * LZ * 8;
    L.xl = o;    o += P * LX * 8;             // one exchange line per pencil (xi_z, then p')
    L.ptile = o; o += 2 * nzpml * P * 8;
    L.spt = o;   o += 2 * nzpml * P * 8;
    L.lines = o; o += 2 * P * LL * 8;         // forward and backward look-back lines per pencil
    o = (o + 15) & ~15;
    L.zs = o;    o += FZ_COUNT * NZP * 4;
    o = (o + 15) & ~15;
    o = (o + 7) & ~7;
    L.mbar = o;  o += 8;                  // mbarrier of the z-table bulk copy
    L.total = (o + 15) & ~15;
    return L;
}

}  // namespace

// P modes per CTA (2, 4 or 8): every pencil's arithmetic is the same for
// each, so the results are too; the launch bounds keep 128 registers per
// thread (P = 8 at W = 2: one 512-thread CTA per SM, the z tables loaded once
// per eight modes).
template <bool D3, int W, int P>
__global__ void __launch_bounds__(P * 64, 8 / P) fused_step_kernel(const FusedArgs A) {
    extern __shared__ __align__(16) unsigned char smraw[];
    constexpr int TP = 32 * W, NZP = TP * CH, LZ = NZP + 2 * GZ, LX = NZP + 2 * GX, LL = TP + 2 * KB;
    constexpr int BCX = D3 ? 1 : 3, BCP = D3 ? 0 : 2;
    const int nz = A.nz, M = A.M, nzpml = A.nzpml, nb = A.npmlbot, nt = A.npmltop;
    const long long fs = A.fs;
    const FusedLayout Ly = fused_layout(P, W, nzpml);
    float2* tile = (float2*)(smraw + Ly.tile);            // [6][P][LZ], level j at GZ + j
    float2* xlb = (float2*)(smraw + Ly.xl);               // [P][LX], level j at GX + j
    float2* ptile = (float2*)(smraw + Ly.ptile);          // [2][nzpml][P]
    float2* spt = (float2*)(smraw + Ly.spt);              // [2][nzpml][P] PML right-hand sides
    float2* lines = (float2*)(smraw + Ly.lines);          // [P][2][LL], chunk t at KB + t
    float* zs = (float*)(smraw + Ly.zs);                  // [FZ_COUNT][NZP]
    const unsigned mbar = (unsigned)__cvta_generic_to_shared(smraw + Ly.mbar);
    const int nthr = blockDim.x;
    const int pi = threadIdx.x / TP;                      // pencil within the CTA
    const int t = threadIdx.x - pi * TP;                  // chunk index
    const int j0 = t * CH;
    float2* xl = xlb + pi * LX + GX;
    float2* lf = lines + (2 * pi) * LL + KB;
    float2* lk = lines + (2 * pi + 1) * LL + KB;
    // work items: (source, group of P modes); CTA b takes items b, b + G, ...
    const int ntile = (M + P - 1) / P;
    const int nitem = ntile * A.nsrc;
    if ((int)blockIdx.x >= nitem) return;           // (the launch never has more CTAs than items)

    // ---- the z tables: one bulk copy (TMA engine) into shared memory, issued
    // by thread 0 and awaited, with a bounded wait, after the cooperative
    // loads below; 16-byte aligned at both ends, a multiple of 16 bytes ----
    if (threadIdx.x == 0) {
        const unsigned bytes = FZ_COUNT * NZP * 4;
        const unsigned dst = (unsigned)__cvta_generic_to_shared(zs);
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(mbar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        if (!A.no_copy) {
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(mbar), "r"(bytes)
                         : "memory");
            asm volatile(
                "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(dst),
                "l"(A.ftab), "r"(bytes), "r"(mbar)
                : "memory");
        }
    }
    // ---- zero the ghost and padding rows of the tile, the exchange lines'
    // ghosts and the look-back lines' end entries ----
    {
        const int nl = LZ - nz;                       // GZ below + (NZP - nz + GZ) above, per row
        for (int r = threadIdx.x; r < 6 * P * nl; r += nthr) {
            const int row = r / nl, k = r - row * nl;
            const int z = k < GZ ? k : nz + k;        // tile index (level z - GZ)
            tile[row * LZ + z] = make_float2(0.f, 0.f);
        }
        for (int r = threadIdx.x; r < P * 2 * GX; r += nthr) {
            const int line = r / (2 * GX), k = r - line * (2 * GX);
            const int z = k < GX ? k : NZP + k;       // ghost entries below 0 and at NZP, NZP+1
            xlb[line * LX + z] = make_float2(0.f, 0.f);
        }
        for (int r = threadIdx.x; r < 2 * P * 2 * KB; r += nthr) {
            const int line = r / (2 * KB), k = r - line * (2 * KB);
            lines[line * LL + (k < KB ? k : TP + k)] = make_float2(0.f, 0.f);
        }
    }
    for (int item = blockIdx.x; item < nitem; item += gridDim.x) {
        const bool first = item == (int)blockIdx.x;
        const int s = item / ntile;
        const int m0 = (item - s * ntile) * P;
        const int m = m0 + pi;
        const bool mvalid = m < M;
        float2* gA = A.a + (long long)s * 6 * fs;
        float2* gS = A.scr + (long long)s * 6 * fs;
        float2* gP = A.pml + (long long)s * 2 * A.ps;
        // 16 B vector copies need every row start z*M + m0 to be even (M even)
        const bool vec = ((M & 1) == 0) && (m0 + P <= M);
        if (!first) {
            // the previous item's update and filter wrote the padding levels
            // nz..NZP-1 of every row: zero them again
            const int np = NZP - nz;
            for (int r = threadIdx.x; r < 6 * P * np; r += nthr) {
                const int row = r / np, k = r - row * np;
                tile[row * LZ + GZ + nz + k] = make_float2(0.f, 0.f);
            }
        }
        // ---- load the a tile and the PML tile: every complex value by its own
        // asynchronous 8-byte copy into its transposed place, all in flight at
        // once ([z][m] in HBM, [mode][z] on chip), awaited with the z tables ----
        {
            constexpr int RPI = TP;                       // rows advanced per pass: blockDim.x / P
            const int q = threadIdx.x % P;
            const bool qv = m0 + q < M;
            const int z0 = threadIdx.x / P;
            if (qv) {
                const unsigned d0 = (unsigned)__cvta_generic_to_shared(tile + q * LZ + GZ + z0);
                const float2* s0 = gA + (long long)z0 * M + m0 + q;
                #pragma unroll 1
                for (int f = 0; f < 6; ++f) {
                    unsigned dst = d0 + f * (P * LZ * 8);
                    size_t src = __cvta_generic_to_global(s0 + f * fs);
                    for (int z = z0; z < nz; z += RPI, dst += RPI * 8, src += (size_t)RPI * M * 8)
                        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(dst), "l"(src) : "memory");
                }
            } else {
                for (int f = 0; f < 6; ++f)
                    for (int z = z0; z < nz; z += RPI) tile[f * P * LZ + q * LZ + GZ + z] = make_float2(0.f, 0.f);
            }
            for (int r = threadIdx.x / P; r < 2 * nzpml; r += RPI) {
                float2* dst = ptile + r * P + q;
                if (qv) {
                    const float2* src = gP + (long long)r * M + m0 + q;
                    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(
                                     (unsigned)__cvta_generic_to_shared(dst)),
                                 "l"(__cvta_generic_to_global(src))
                                 : "memory");
                } else {
                    *dst = make_float2(0.f, 0.f);
                }
            }
        }
        const int tl = *A.clk.time - A.clk.t0[s];           // this slot's clock
        const bool src_on = A.src_mode != 0 && slot_src_on(A.clk, tl);
        // this mode's multipliers, loaded while the tile copies are in flight
        const float kx = mvalid ? A.pt[PT_KX * M + m] : 0.f;
        const float ky = mvalid ? A.pt[PT_KY * M + m] : 0.f;
        const float gd = (mvalid && A.damp) ? A.pt[PT_DAMP * M + m] : 0.f;
        asm volatile("cp.async.wait_all;\n" ::: "memory");
        __syncthreads();                                      // the tiles are in, the mbarrier is initialised
        // bounded wait for the tables; if it gives up anywhere in the CTA, the CTA
        // reports it and leaves without computing or storing (its modes keep the
        // state of the previous step), thread 0 first waiting out a copy still in
        // flight so that nothing lands in shared memory after the CTA has gone
        if (first && __syncthreads_or(!mbar_wait(mbar, A.wait_limit))) {
            if (threadIdx.x == 0) {
                atomicExch(A.err, 1);
                if (!A.no_copy) mbar_wait(mbar, 1 << 22);
            }
            return;
        }

        // ---- L2 prefetch of the rows of the CTA that starts pf_stride CTAs
        // later (about when this one ends): its tile load then comes from L2 ----
        if (A.pf_stride > 0) {
            const int nid = item + gridDim.x;             // this CTA's next item
            if (nid < nitem) {
                const int ns = nid / ntile, nm0 = (nid - ns * ntile) * P;
                const float2* nA = A.a + (long long)ns * 6 * fs + nm0;
                for (int r = threadIdx.x; r < 6 * nz; r += nthr) {
                    const int f = r / nz, z = r - f * nz;
                    const float2* row = nA + f * fs + (long long)z * M;
                    asm volatile("prefetch.global.L2 [%0];" ::"l"(__cvta_generic_to_global(row)));
                }
                const float2* nP = A.pml + (long long)ns * 2 * A.ps + nm0;
                for (int r = threadIdx.x; r < 2 * nzpml; r += nthr)
                    asm volatile("prefetch.global.L2 [%0];" ::"l"(__cvta_generic_to_global(nP + (long long)r * M)));
            }
        }

        const float2 NGD = bc2(-gd);
        // threads that own rows with special rules
        const bool lo = (j0 == 0);                                       // rows 0, 1
        const bool hi = (j0 <= nz - 1) && (j0 + CH > nz - 2);            // rows nz-2, nz-1
        // PML levels of this chunk: bit q of pmask, plane index pipv + q (a chunk
        // holds contiguous levels of one layer at most)
        unsigned pmask = 0;
        int pipv = 0;
        if (j0 < nb) {
            pmask = (1u << min(CH, nb - j0)) - 1u;
            pipv = j0;
        } else {
            const int l0 = max(j0, nz - nt), l1 = min(j0 + CH, nz);
            if (l1 > l0) {
                pmask = ((1u << (l1 - l0)) - 1u) << (l0 - j0);
                pipv = nb + (j0 - (nz - nt));
            }
        }
        const bool pml_t = pmask != 0;
        const bool src_t = src_on && mvalid && A.ksrc >= j0 && A.ksrc < j0 + CH;
        // forcing of this step for this mode (only the thread owning the source plane uses it)
        float2 F = make_float2(0.f, 0.f);
        if (src_t) {
            if (A.src_mode == 1) {
                const float2* pl = A.planes + (long long)s * A.plane_ss + m;
                float w = (tl < A.nseries) ? (float)A.series[(long long)s * A.nseries + tl] : 0.f;
                F = w * pl[0];
            } else {   // this step's interpolated plane, from source_plane_kernel
                F = A.src_plane[(long long)s * M + m];
            }
            F = A.src_scale * F;
        }

        float2 sc[6][CH];
        #pragma unroll
        for (int f = 0; f < 6; ++f)
            #pragma unroll
            for (int q = 0; q < CH; ++q) sc[f][q] = make_float2(0.f, 0.f);

        float2* tp = tile + pi * LZ + GZ;                    // field f, level j: tp[f*P*LZ + j]
        auto TA = [&](int f, int j) -> float2 { return tp[f * P * LZ + j]; };
        // z table entry of row r at level j, as a pair
        auto Z2 = [&](int r, int j) { return zt2(zs, r * NZP + j); };

        // one LDDRK stage; HS: the stage argument is a + beta*scr (stages 2-5)
        // rather than a (stage 1), fixed at compile time
        auto stage = [&](auto hs_c, const float beta) {
            constexpr bool hs = decltype(hs_c)::value;
            const float2 BT = bc2(beta);
            // ---- temp xi_z into the first exchange line ----
            float2 own[CH];
            #pragma unroll
            for (int q = 0; q < CH; ++q) {
                float2 v = TA(2, j0 + q);
                if (hs) v = pfma(BT, sc[2][q], v);
                own[q] = v;
                // level j0+2 is no neighbour's stencil value; only the top rows'
                // closure (levels nz-5..nz-1) may read it from the line
                if (q != 2 || j0 + 2 >= nz - 5) xl[j0 + q] = v;
            }
            float2 top = make_float2(0.f, 0.f);
            if (!D3 && hi) {   // caller-set top value of bc 3 (physics2d.f90:960)
                float2 last = make_float2(0.f, 0.f);
                #pragma unroll
                for (int q = 0; q < CH; ++q)
                    if (j0 + q == nz - 1) last = sc[0][q];
                float2 xx = TA(0, nz - 1);
                if (hs) xx = xx + beta * last;
                top = -(imul(kx, xx) * A.unstr_top);
            }
            pencil_sync(pi, TP);
            float2 d[CH];
            // d: the stretched derivative (the solve's tables carry the stretch)
            zsolve<BCX, W>(xl, own, zs, FZ_SX, FZ_LX, nz, top, j0, lo, hi, t, lf, lk, pi, A.cc, d);
            if (pml_t) {   // psi_vz (displacement.f90 PML rows)
                #pragma unroll
                for (int q = 0; q < CH; ++q) {
                    if (pmask & (1u << q)) {
                        const int j = j0 + q, ip = pipv + q;
                        float2 psi = ptile[ip * P + pi];
                        if (hs) psi = psi + beta * spt[ip * P + pi];
                        spt[ip * P + pi] = Z2(FZ_AZ, j).x * d[q] + Z2(FZ_BZ, j).x * psi;
                        d[q] = d[q] + psi;
                    }
                }
            }
            // ---- div, p', the buoyancy term, horizontal right-hand sides ----
            float2 qt[CH];
            #pragma unroll
            for (int q = 0; q < CH; ++q) {
                const int j = j0 + q;
                float2 xx = TA(0, j);
                const float2 xz = own[q];      // the xi_z stage argument, still in registers
                if (hs) xx = pfma(BT, sc[0][q], xx);
                float2 div = imul(kx, xx) + d[q];
                if (D3) {
                    float2 xy = TA(1, j);
                    if (hs) xy = pfma(BT, sc[1][q], xy);
                    div = div + imul(ky, xy);
                }
                const float2 p = pmul(make_float2(-1.f, -1.f), pfma(Z2(FZ_GP, j), xz, pmul(Z2(FZ_C2R, j), div)));
                qt[q] = pfma(Z2(FZ_E2, j), xz, pmul(Z2(FZ_E1, j), div));   // -g rho'/rho0
                if (q != 2 || j0 + 2 >= nz - 5) xl[j] = p;
                own[q] = p;
            }
            pencil_sync(pi, TP);
            // ---- dp'/dz, RHS v_z and xi_z ----
            // d: (stretch / rho0) dp'/dz, scaled by the solve's tables
            zsolve<BCP, W>(xl, own, zs, FZ_SP, FZ_LP, nz, make_float2(0.f, 0.f), j0, lo, hi, t, lf, lk, pi, A.cc, d);
            // ---- horizontal right-hand sides (they do not feed the p' solve) ----
            #pragma unroll
            for (int q = 0; q < CH; ++q) {
                const int j = j0 + q;
                float2 vx = TA(3, j);
                if (hs) vx = pfma(BT, sc[3][q], vx);
                const float ri = Z2(FZ_RI, j).x;
                sc[3][q] = pfma(NGD, vx, -ri * imul(kx, own[q]));
                sc[0][q] = vx;
                if (D3) {
                    float2 vy = TA(4, j);
                    if (hs) vy = pfma(BT, sc[4][q], vy);
                    sc[4][q] = pfma(NGD, vy, -ri * imul(ky, own[q]));
                    sc[1][q] = vy;
                }
            }
            // zero right-hand side rows: j = 0 (and j = nz-1 in 3-D)
            if (lo) { sc[3][0] = sc[0][0] = make_float2(0.f, 0.f); if (D3) sc[4][0] = sc[1][0] = sc[3][0]; }
            if (D3 && hi) {
                #pragma unroll
                for (int q = 0; q < CH; ++q)
                    if (j0 + q == nz - 1) sc[0][q] = sc[1][q] = sc[3][q] = sc[4][q] = make_float2(0.f, 0.f);
            }
            #pragma unroll
            for (int q = 0; q < CH; ++q) {
                const int j = j0 + q;
                float2 vz = TA(5, j);
                if (hs) vz = pfma(BT, sc[5][q], vz);
                sc[5][q] = pfma(NGD, vz, psub(qt[q], d[q]));
                sc[2][q] = vz;
            }
            if (pml_t) {   // psi_p
                #pragma unroll
                for (int q = 0; q < CH; ++q) {
                    if (pmask & (1u << q)) {
                        const int j = j0 + q, ip = pipv + q;
                        float2 psi = ptile[(nzpml + ip) * P + pi];
                        if (hs) psi = psi + beta * spt[(nzpml + ip) * P + pi];
                        spt[(nzpml + ip) * P + pi] = Z2(FZ_AZR, j).x * d[q] + Z2(FZ_BZ, j).x * psi;
                        sc[5][q] = sc[5][q] - Z2(FZ_RI, j).x * psi;
                    }
                }
            }
            if (src_t) {
                #pragma unroll
                for (int q = 0; q < CH; ++q)
                    if (j0 + q == A.ksrc) sc[5][q] = sc[5][q] + F;
            }
            if (lo) sc[5][0] = sc[2][0] = make_float2(0.f, 0.f);
            if (D3 && hi) {
                #pragma unroll
                for (int q = 0; q < CH; ++q)
                    if (j0 + q == nz - 1) sc[5][q] = sc[2][q] = make_float2(0.f, 0.f);
            }
        };
        stage(std::integral_constant<bool, false>(), 0.f);
        for (int rk = 1; rk < 5; ++rk) {
            // static parameter indices keep the argument block out of local memory
            const float beta = rk == 1 ? A.betas[1] : rk == 2 ? A.betas[2] : rk == 3 ? A.betas[3] : A.betas[4];
            stage(std::integral_constant<bool, true>(), beta);
        }

        // ---- update a += dt*scr, pml += dt*scrpml (step.f90:114-116) ----
        const float dt = A.dt;
        const float2 DT = bc2(dt);
        #pragma unroll
        for (int f = 0; f < 6; ++f)
            #pragma unroll
            for (int q = 0; q < CH; ++q) {
                float2* a = tp + f * P * LZ + j0 + q;
                *a = pfma(DT, sc[f][q], *a);
            }
        if (pml_t) {
            #pragma unroll
            for (int q = 0; q < CH; ++q) {
                if (pmask & (1u << q)) {
                    const int ip = pipv + q;
                    ptile[ip * P + pi] = ptile[ip * P + pi] + dt * spt[ip * P + pi];
                    ptile[(nzpml + ip) * P + pi] = ptile[(nzpml + ip) * P + pi] + dt * spt[(nzpml + ip) * P + pi];
                }
            }
        }
        pencil_sync(pi, TP);
        // ---- z filter (+ horizontal filter): field f is filtered into registers,
        // and written back after the next barrier, while field f+1 is filtered ----
        const float hf = mvalid ? A.pt[PT_HF * M + m] : 1.f;
        const float h1 = 0.5f * 0.41015625f, h2 = 0.5f * -0.234375f, h3 = 0.5f * 0.087890625f;
        const float h4 = 0.5f * -0.01953125f, h5 = 0.5f * 0.001953125f, c0 = 0.75390625f;
        const bool hfil_on = slot_hfilter(A.clk, tl);
        const bool flo = j0 < 5, fhi = (j0 < nz) && (j0 + CH > nz - 5);
        float2 prev[CH];
        #pragma unroll
        for (int f = 0; f < 7; ++f) {
            float2 out[CH];
            if (f < 6) {
                const float2* V = tp + f * P * LZ;
                #pragma unroll
                for (int q = 0; q < CH; ++q) {
                    const int j = j0 + q;
                    float2 acc = pmul(bc2(c0), V[j]);
                    acc = pfma(bc2(h1), padd(V[j - 1], V[j + 1]), acc);
                    acc = pfma(bc2(h2), padd(V[j - 2], V[j + 2]), acc);
                    acc = pfma(bc2(h3), padd(V[j - 3], V[j + 3]), acc);
                    acc = pfma(bc2(h4), padd(V[j - 4], V[j + 4]), acc);
                    out[q] = pfma(bc2(h5), padd(V[j - 5], V[j + 5]), acc);
                }
                if (flo || fhi) {   // FILTER_VARS_3D / _2D boundary rows
                    #pragma unroll
                    for (int q = 0; q < CH; ++q) {
                        const int j = j0 + q;
                        const bool near_bot = (j >= 1 && j <= 4), near_top = (j >= nz - 5 && j <= nz - 2);
                        if (j == 0 || j == nz - 1) out[q] = V[j];
                        else if (near_top) out[q] = 0.5f * (V[j + 1] + V[j - 1]);
                        else if (near_bot) out[q] = D3 ? 0.5f * (V[j + 1] + V[j - 1]) : V[j];
                    }
                }
                if (hfil_on && (D3 ? (f < 5) : true)) {
                    #pragma unroll
                    for (int q = 0; q < CH; ++q) out[q] = hf * out[q];
                }
            }
            if (f > 0) {
                pencil_sync(pi, TP);   // every thread has read field f-1's neighbours
                #pragma unroll
                for (int q = 0; q < CH; ++q) tp[(f - 1) * P * LZ + j0 + q] = prev[q];
            }
            #pragma unroll
            for (int q = 0; q < CH; ++q) prev[q] = out[q];
        }
        __syncthreads();   // the store below copies every pencil's rows
        // ---- store a and the PML planes.  A row [f][z] of the CTA's P modes is
        // 8P contiguous bytes in HBM; P/2 consecutive lanes write it as P/2
        // float4, so every warp store covers whole rows (full sectors) instead
        // of 16 bytes in each of 32 rows ----
        constexpr int LPR = P / 2;                            // lanes per row
        const int lq = threadIdx.x % LPR;                     // this lane's modes: 2 lq, 2 lq + 1
        auto store_rows = [&](float2* gbase) {
            #pragma unroll 1
            for (int f = 0; f < 6; ++f) {
                for (int z = threadIdx.x / LPR; z < nz; z += nthr / LPR) {
                    float2* dst = gbase + f * fs + (long long)z * M + m0 + 2 * lq;
                    const float2* srcp = tile + f * P * LZ + (2 * lq) * LZ + GZ + z;
                    if (vec) {
                        const float2 w0 = srcp[0], w1 = srcp[LZ];
                        *(float4*)dst = make_float4(w0.x, w0.y, w1.x, w1.y);
                    } else {
                        if (m0 + 2 * lq < M) dst[0] = srcp[0];
                        if (m0 + 2 * lq + 1 < M) dst[1] = srcp[LZ];
                    }
                }
            }
        };
        store_rows(gA);
        for (int r = threadIdx.x / LPR; r < 2 * nzpml; r += nthr / LPR) {
            float2* dst = gP + (long long)r * M + m0 + 2 * lq;
            const float2* srcp = ptile + r * P + 2 * lq;
            if (vec) {
                *(float4*)dst = *(const float4*)srcp;
            } else {
                if (m0 + 2 * lq < M) dst[0] = srcp[0];
                if (m0 + 2 * lq + 1 < M) dst[1] = srcp[1];
            }
        }
        // ---- the last stage's right-hand side, when an output needs it ----
        if (A.write_scr) {
            __syncthreads();
            #pragma unroll
            for (int f = 0; f < 6; ++f)
                #pragma unroll
                for (int q = 0; q < CH; ++q) tp[f * P * LZ + j0 + q] = sc[f][q];
            __syncthreads();
            store_rows(gS);
        }
        // every thread has read the tile and the PML tile out for the stores
        // (in flight now) before the next item's copies overwrite them
        __syncthreads();
    }
}

// LAGRANGE_INTERP source of the fused step (physics.f90:683-734): the plane
// of every slot interpolated to the step about to run, sum over l of
// w(l) * vr(l) with the FP64 weights of the slot's clock (samples that take
// no part have weight 0 and are skipped), in FP32 in the order of l.  One
// launch before each fused step, so that the step's CTAs read one value
// instead of each computing the seven FP64 weights on its critical path.
__global__ void __launch_bounds__(256) source_plane_kernel(const FusedArgs A) {
    __shared__ double w[8];
    __shared__ int id[8];
    const int s = blockIdx.y;
    if (threadIdx.x < 7) {
        const int tl = *A.clk.time - A.clk.t0[s];
        int i;
        const double v = lagrange_weight(A.clk, tl, A.L, threadIdx.x, &i);
        w[threadIdx.x] = v;
        id[threadIdx.x] = i < 0 ? 0 : i;
    }
    __syncthreads();
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= A.M) return;
    const float2* pl = A.planes + (long long)s * A.plane_ss + m;
    float2 F = make_float2(0.f, 0.f);
    #pragma unroll
    for (int l = 0; l < 7; ++l)
        if (w[l] != 0.0) F = F + (float)w[l] * pl[(long long)id[l] * A.M];
    A.src_plane[(long long)s * A.M + m] = F;
}

void launch_source_plane(const FusedArgs& A, int nsrc, cudaStream_t s) {
    source_plane_kernel<<<dim3((A.M + 255) / 256, nsrc), 256, 0, s>>>(A);
}

int fused_w(int nz) { return (nz + 32 * CH - 1) / (32 * CH); }
int fused_nzp(int nz) { return 32 * CH * fused_w(nz); }

// whether P modes per CTA fit the 227 KB of shared memory a CTA may use
bool fused_fits(int P, int nz, int nzpml) {
    return fused_layout(P, fused_w(nz), nzpml).total <= 227 * 1024;
}

size_t fused_smem_bytes(int nz, int nzpml, int W) {
    (void)nz;
    return (size_t)fused_layout(4, W, nzpml).total;
}

// nz >= 16 keeps the boundary rows of the two ends in different threads
int fused_supported(int nz) { return nz >= 16 && nz <= 2 * 32 * CH; }

template <bool D3, int W, int P>
static void fused_attr(int nzpml) {
    const size_t sm = (size_t)fused_layout(P, W, nzpml).total;
    cudaFuncSetAttribute((const void*)fused_step_kernel<D3, W, P>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)sm);
}

// Dynamic shared-memory limits of every variant a context may launch, set
// once at context creation (not while a launch sequence is being captured).
void fused_prepare(int nz, int nzpml) {
    const int W = fused_w(nz);
    if (W == 1) {
        fused_attr<true, 1, 2>(nzpml); fused_attr<true, 1, 4>(nzpml); fused_attr<true, 1, 8>(nzpml);
        fused_attr<false, 1, 2>(nzpml); fused_attr<false, 1, 4>(nzpml); fused_attr<false, 1, 8>(nzpml);
    } else {
        fused_attr<true, 2, 2>(nzpml); fused_attr<true, 2, 4>(nzpml); fused_attr<true, 2, 8>(nzpml);
        fused_attr<false, 2, 2>(nzpml); fused_attr<false, 2, 4>(nzpml); fused_attr<false, 2, 8>(nzpml);
    }
}

template <bool D3, int W, int P>
static void launch_fused_t(const FusedArgs& A, int nsrc, cudaStream_t s) {
    const size_t sm = (size_t)fused_layout(P, W, A.nzpml).total;
    FusedArgs B = A;
    B.nsrc = nsrc;
    int dev = 0, nsm = 0, occ = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fused_step_kernel<D3, W, P>, P * 32 * W, sm);
    const long long items = (long long)((A.M + P - 1) / P) * nsrc;
    const long long resident = (long long)std::max(nsm, 1) * std::max(occ, 1);
    const int ncta = (int)std::min(items, resident);
    fused_step_kernel<D3, W, P><<<ncta, P * 32 * W, sm, s>>>(B);
}

template <bool D3, int W>
static void launch_fused_p(const FusedArgs& A, int nsrc, cudaStream_t s) {
    if (A.pencils == 2) launch_fused_t<D3, W, 2>(A, nsrc, s);
    else if (A.pencils == 8) launch_fused_t<D3, W, 8>(A, nsrc, s);
    else launch_fused_t<D3, W, 4>(A, nsrc, s);
}

void launch_fused(const FusedArgs& A, int nsrc, cudaStream_t s) {
    const bool d3 = (A.option == 4);
    if (A.W == 1) {
        if (d3) launch_fused_p<true, 1>(A, nsrc, s); else launch_fused_p<false, 1>(A, nsrc, s);
    } else {
        if (d3) launch_fused_p<true, 2>(A, nsrc, s); else launch_fused_p<false, 2>(A, nsrc, s);
    }
}
