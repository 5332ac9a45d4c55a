// C-ABI implementation of include/sparc_gpu.h: context life cycle, the FP64
// host set-up that replaces the reference's initialisation routines, the
// TIMESTEPPING loop body, state transfer, surface recording, sensitivity
// kernels and checkpointing.  All device work runs on the context's stream.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include <algorithm>

#include "ctx.cuh"
#include "adjsrc.cuh"
#include "update.cuh"

namespace {


// ---------------------------------------------------------------------------
// compact finite differences on the host (set-up only): DBYD2 / MTRIDAG
// ---------------------------------------------------------------------------
struct Tri {
    std::vector<double> low, upp, betad, gam;
};

void compact_coeffs(int nz, Compact<double>& cc) {
    double d2i = (double)(float)(nz - 1);                       // dbyd2.f90:49
    cc.C1 = d2i * 7.0 / 9.0;                                    // dbyd2.f90:88
    cc.C2 = d2i / 36.0;
    cc.Cb[0] = -(double)(43.0f / 96.0f) * d2i;                  // dbyd2.f90:104-108 (REAL*4 ratios)
    cc.Cb[1] = -(double)(5.0f / 6.0f) * d2i;
    cc.Cb[2] = (double)(9.0f / 8.0f) * d2i;
    cc.Cb[3] = (double)(1.0f / 6.0f) * d2i;
    cc.Cb[4] = -(double)(1.0f / 96.0f) * d2i;
    cc.Cf[0] = -(double)(10.0f / 3.0f) * d2i;                   // dbyd2.f90:122-125
    cc.Cf[1] = -3.0 * d2i;
    cc.Cf[2] = 6.0 * d2i;
    cc.Cf[3] = (double)(1.0f / 3.0f) * d2i;
    cc.alpha2 = 0.75;                                           // dbyd2.f90:157-162
    cc.beta1 = 3.0;
    cc.cnst = 1.0 / (0.75 - 3.0 * 0.125);
}

// matrix of DBYD2 for boundary code ibc (dbyd2.f90:152-196) and its Thomas
// factorisation (mtridag.f90:95-99)
Tri tri_for(int nz, int ibc) {
    Tri t;
    std::vector<double> uppr(nz + 1, 0.0), lowr(nz + 1, 0.0);
    double alpha = (double)(1.0f / 3.0f);
    for (int J = 3; J <= nz - 2; ++J) uppr[J] = alpha;
    double alpha2 = 0.75, gamma2 = 0.125, alpha1 = 6.0, beta1 = 3.0;
    double cnst = 1.0 / (alpha2 - beta1 * gamma2);
    double up1 = (alpha1 * alpha2 - beta1) * cnst;
    uppr[1] = (ibc % 2 == 0) ? 0.0 : up1;
    uppr[2] = alpha2;
    uppr[nz - 1] = gamma2;
    for (int I = 1; I <= nz; ++I) lowr[I] = uppr[nz - I + 1];
    lowr[nz] = (ibc != 1 && ibc != 2) ? 0.0 : up1;
    t.low.assign(lowr.begin() + 1, lowr.end());
    t.upp.assign(uppr.begin() + 1, uppr.end());
    t.betad.assign(nz, 0.0);
    t.gam.assign(nz, 0.0);
    t.betad[0] = 1.0;
    for (int J = 1; J < nz; ++J) {
        t.gam[J] = t.upp[J - 1] / t.betad[J - 1];
        t.betad[J] = 1.0 - t.low[J] * t.gam[J];
    }
    return t;
}

// Elimination rows of the fused step for boundary code ibc (FP64): 1/betad,
// the forward multipliers m, their products H from each chunk's first level,
// the backward multipliers g and their products G from each chunk's last
// level (chunks of FUSED_CH levels; padding levels up to nzp are zero).
struct FusedRows {
    std::vector<double> ibd, mm, HH, gg, GG;
};
FusedRows fused_rows(int nz, int nzp, const Tri& t) {
    FusedRows r;
    r.ibd.assign(nzp, 0.0); r.mm.assign(nzp, 0.0); r.gg.assign(nzp, 0.0); r.HH.assign(nzp, 0.0);
    r.GG.assign(nzp, 0.0);
    for (int j = 0; j < nz; ++j) {
        r.ibd[j] = 1.0 / t.betad[j];
        r.mm[j] = (j == 0) ? 0.0 : -t.low[j] / t.betad[j];
        r.gg[j] = (j == nz - 1) ? 0.0 : -t.gam[j + 1];
    }
    for (int j0 = 0; j0 < nzp; j0 += FUSED_CH) {
        const int j1 = j0 + FUSED_CH;
        double pr = 1.0;
        for (int j = j0; j < j1; ++j) { pr *= r.mm[j]; r.HH[j] = pr; }
        pr = 1.0;
        for (int j = j1 - 1; j >= j0; --j) { pr *= r.gg[j]; r.GG[j] = pr; }
    }
    return r;
}

// The elimination rows of the same solve for y(j) = sig(j) x(j): forward
// variable sig(j) u(j), so 1/betad -> sig(j)/betad(j) and m(j) -> m(j)
// sig(j)/sig(j-1); back substitution y(j) = sig(j) u(j) + g(j) sig(j)/sig(j+1)
// y(j+1); the chunk products H, G are those of the new multipliers.  Same
// recurrences, the scale applied inside them (sig = 1 on padding levels).
FusedRows fused_rows_scaled(const FusedRows& r, const std::vector<double>& sig) {
    FusedRows o = r;
    const int nzp = (int)r.ibd.size();
    for (int j = 0; j < nzp; ++j) {
        o.ibd[j] = r.ibd[j] * sig[j];
        o.mm[j] = (j == 0) ? r.mm[j] : r.mm[j] * sig[j] / sig[j - 1];
        o.gg[j] = (j == nzp - 1) ? r.gg[j] : r.gg[j] * sig[j] / sig[j + 1];
    }
    for (int j0 = 0; j0 < nzp; j0 += FUSED_CH) {
        const int j1 = j0 + FUSED_CH;
        double pr = 1.0;
        for (int j = j0; j < j1; ++j) { pr *= o.mm[j]; o.HH[j] = pr; }
        pr = 1.0;
        for (int j = j1 - 1; j >= j0; --j) { pr *= o.gg[j]; o.GG[j] = pr; }
    }
    return o;
}

// The fused step's carry table K: the response of the chunk's back
// substitution (zero carry from above) to the carry uin from below,
// K(j) = H(j) + g(j) K(j+1) within the chunk, K(last) = H(last).  The rows
// keep H's place; the look-back products use H itself.
std::vector<double> fused_k_row(const FusedRows& r) {
    const int nzp = (int)r.HH.size();
    std::vector<double> K(nzp, 0.0);
    for (int j0 = 0; j0 < nzp; j0 += FUSED_CH) {
        const int j1 = j0 + FUSED_CH;
        K[j1 - 1] = r.HH[j1 - 1];
        for (int j = j1 - 2; j >= j0; --j) K[j] = r.HH[j] + r.gg[j] * K[j + 1];
    }
    return K;
}

// Look-back products of the fused step's carries: fwd[4t + i-2] is the
// product of the chunk multipliers Mc(t-1)..Mc(t-i+1) (i = 2..5), the factor
// of chunk t-i's value in the carry into chunk t; bwd[4t + i-2] likewise with
// the backward chunk multipliers Gc(t+1)..Gc(t+i-1) for chunk t+i.  Returns
// the largest product over FUSED_KB chunks, the factor of the first chunk the
// carries leave out, over the chunks that hold real levels (the carries into
// padding chunks reach no real row: their H and G rows are zero).
double fused_lookback(const FusedRows& r, int tp, int nz, std::vector<double>& fwd, std::vector<double>& bwd) {
    std::vector<double> Mc(tp), Gc(tp);
    for (int t = 0; t < tp; ++t) {
        Mc[t] = r.HH[t * FUSED_CH + FUSED_CH - 1];
        Gc[t] = r.GG[t * FUSED_CH];
    }
    fwd.assign((size_t)4 * tp, 0.0);
    bwd.assign((size_t)4 * tp, 0.0);
    double worst = 0.0;
    for (int t = 0; t < tp; ++t) {
        double pf = 1.0, pb = 1.0;
        for (int i = 2; i <= FUSED_KB + 1; ++i) {
            pf = (t - i + 1 >= 0) ? pf * Mc[t - i + 1] : 0.0;
            pb = (t + i - 1 < tp) ? pb * Gc[t + i - 1] : 0.0;
            if (i <= FUSED_KB) {
                fwd[(size_t)4 * t + i - 2] = pf;
                bwd[(size_t)4 * t + i - 2] = pb;
            } else if (t * FUSED_CH < nz) {
                worst = std::max(worst, std::max(std::fabs(pf), std::fabs(pb)));
            }
        }
    }
    return worst;
}

// Whether the look-back carries of the fused step are exact to the stated
// bound for the two boundary codes of a form (xi_z and p')
bool fused_lookback_ok(int nz, int bcx, int bcp) {
    const int nzp = fused_nzp(nz), tp = nzp / FUSED_CH;
    for (int b : {bcx, bcp}) {
        std::vector<double> f, g;
        if (fused_lookback(fused_rows(nz, nzp, tri_for(nz, b)), tp, nz, f, g) > FUSED_LOOKBACK_BOUND) return false;
    }
    return true;
}

// ddz of one z-profile (dbyd2 + stretch), divisions as in mtridag.f90:100-107
void host_dbyd2(const std::vector<double>& b, std::vector<double>& a, int ibc, const Compact<double>& cc,
                const Tri& t) {
    int n = (int)b.size();
    std::vector<double> R(n, 0.0);
    for (int j = 2; j <= n - 3; ++j) R[j] = cc.C1 * (b[j + 1] - b[j - 1]) + cc.C2 * (b[j + 2] - b[j - 2]);
    R[1] = cc.Cb[0] * b[0] + cc.Cb[1] * b[1] + cc.Cb[2] * b[2] + cc.Cb[3] * b[3] + cc.Cb[4] * b[4];
    R[n - 2] = -(cc.Cb[0] * b[n - 1] + cc.Cb[1] * b[n - 2] + cc.Cb[2] * b[n - 3] + cc.Cb[3] * b[n - 4] + cc.Cb[4] * b[n - 5]);
    R[0] = (ibc == 1 || ibc == 3) ? cc.Cf[0] * b[0] + cc.Cf[1] * b[1] + cc.Cf[2] * b[2] + cc.Cf[3] * b[3] : 0.0;
    R[n - 1] = (ibc == 1 || ibc == 2)
                   ? -(cc.Cf[0] * b[n - 1] + cc.Cf[1] * b[n - 2] + cc.Cf[2] * b[n - 3] + cc.Cf[3] * b[n - 4])
                   : 0.0;
    if (ibc % 2 != 0) R[0] = (cc.alpha2 * R[0] - cc.beta1 * R[1]) * cc.cnst;
    if (ibc == 1 || ibc == 2) R[n - 1] = (cc.alpha2 * R[n - 1] - cc.beta1 * R[n - 2]) * cc.cnst;
    std::vector<double> ud(n);
    ud[0] = R[0] / t.betad[0];
    for (int J = 1; J < n; ++J) ud[J] = (R[J] - t.low[J] * ud[J - 1]) / t.betad[J];
    for (int J = n - 2; J >= 0; --J) ud[J] = ud[J] - t.gam[J + 1] * ud[J + 1];
    a = ud;
}



}  // namespace

void sparc_internal_xform_info(const sparc_ctx* c, SparcXformInfo* out) {
    out->nx = c->P.nx;
    out->ny = c->P.ny;
    out->M = c->M;
    out->f32 = c->f32;
    out->tw_x = c->tw_x;
    out->tw_y = c->tw_y;
    out->stream = c->stream;
}
void sparc_internal_set_error(sparc_ctx* c, const std::string& msg) { c->err = msg; }
void sparc_internal_count_launches(sparc_ctx* c, int n) { c->launches += n; }

// ===========================================================================
extern "C" {

int sparc_gpu_abi_version(void) { return SPARC_GPU_ABI_VERSION; }

const char* sparc_gpu_errstr(int s) {
    switch (s) {
        case SPARC_OK: return "ok";
        case SPARC_EINVAL: return "invalid argument or parameter";
        case SPARC_ENOMEM: return "out of memory";
        case SPARC_ECUDA: return "CUDA error";
        case SPARC_ETIMEDOUT: return "device wait timed out";
        case SPARC_ENAN: return "non-finite value in the state";
        case SPARC_ESTATE: return "call out of order";
        case SPARC_EIO: return "file I/O error or corrupt checkpoint";
        default: return "unknown status";
    }
}

const char* sparc_gpu_last_error(const sparc_ctx* c) { return c ? c->err.c_str() : "null context"; }

static int validate(const sparc_params* p, std::string& why) {
    auto pow2 = [](int n) { return n >= 4 && n <= 1024 && (n & (n - 1)) == 0; };
    if (p->option != 2 && p->option != 4 && p->option != 8 && p->option != 10 && p->option != 17 && p->option != 18) {
        why = "option must be 2, 4, 8, 10, 17 or 18";
        return 0;
    }
    if (!pow2(p->nx)) { why = "nx must be a power of two in [4,1024]"; return 0; }
    const bool is2d = (p->option == 17 || p->option == 18);
    if (is2d && p->ny != 1) { why = "the 2-D options (17, 18) need ny == 1"; return 0; }
    if (!is2d && !pow2(p->ny)) { why = "ny must be a power of two in [4,1024]"; return 0; }
    if (p->nz < 16 || p->nz > 1024) { why = "nz must be in [16,1024]"; return 0; }
    if (p->npmlbot < 2 || p->npmlbot > p->nz / 4 || p->npmltop < 0 || p->npmltop > p->nz / 4) {
        why = "PML widths out of range"; return 0;
    }
    if (p->precision != SPARC_FP64 && p->precision != SPARC_FP32) { why = "bad precision"; return 0; }
    if (p->nsrc < 1 || p->nsrc > 4096) { why = "nsrc out of range"; return 0; }
    if (!(p->timestep > 0) || !(p->xlength > 0) || !(p->ylength > 0) || !(p->cadforcing > 0) || !(p->outputcad > 0)) {
        why = "lengths and times must be positive"; return 0;
    }
    if (p->src_k < 0 || p->src_k > p->nz) { why = "src_k out of range"; return 0; }
    return 1;
}

int sparc_gpu_create(const sparc_params* p, sparc_ctx** out) {
    if (!out) return SPARC_EINVAL;
    *out = nullptr;
    if (!p) return SPARC_EINVAL;
    std::string why;
    if (!validate(p, why)) return SPARC_EINVAL;
    sparc_ctx* c = new sparc_ctx();
    c->P = *p;
    c->H = p->nx / 2 + 1;
    c->M = p->ny * c->H;
    c->nz = p->nz;
    c->S = p->nsrc;
    c->nzpml = p->npmlbot + p->npmltop;
    c->fs = (long long)c->nz * c->M;
    c->ps = (long long)std::max(c->nzpml, 1) * c->M;
    c->NP = (long long)p->nx * p->ny;
    c->N = c->NP * c->nz;
    c->f32 = (p->precision == SPARC_FP32);
    c->nf = (p->option == 8) ? 8 : 6;            // dimfive: rho, v, p, b in the MHD velocity form
    const bool mhd_form = (p->option == 8 || p->option == 10 || p->option == 18);
    int rc = SPARC_OK;
    auto bail = [&](int code) { sparc_gpu_destroy(c); return code; };
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_done, cudaEventDisableTiming) != cudaSuccess) {
        cudaGetLastError();
        if (c->stream) cudaStreamDestroy(c->stream);
        delete c;
        return SPARC_ECUDA;
    }
    size_t cs = csz(c), es = esz(c);
    long long S = c->S;
    if ((rc = dalloc(c, &c->a, (size_t)S * c->nf * c->fs * cs))) return bail(rc);
    if ((rc = dalloc(c, &c->scr, (size_t)S * c->nf * c->fs * cs))) return bail(rc);
    if ((rc = dalloc(c, &c->pml, (size_t)S * 2 * c->ps * cs))) return bail(rc);
    if ((rc = dalloc(c, &c->scrpml, (size_t)S * 2 * c->ps * cs))) return bail(rc);
    if ((rc = dalloc(c, &c->ybuf, (size_t)S * c->fs * cs))) return bail(rc);
    if ((rc = dalloc(c, &c->pbuf, (size_t)S * c->fs * cs))) return bail(rc);
    if ((rc = dalloc(c, &c->rbuf, (size_t)S * c->fs * cs))) return bail(rc);
    if ((rc = dalloc(c, &c->zt, (size_t)ZT_COUNT * c->nz * es))) return bail(rc);
    if ((rc = dalloc(c, &c->pt, (size_t)PT_COUNT * c->M * es))) return bail(rc);
    {
        // per-stage kernels run one thread per (mode, source): the default CTA
        // is the largest of 128, 64, 32 threads whose grid still gives every
        // SM two CTAs (small grids, e.g. 128x128 with 8320 modes, need 32)
        int dev = 0, nsm = 152;
        if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        cudaGetLastError();
        // FP64 quiet displacement forms: lanes per pencil (stage_chunk_kernel
        // and update_chunk_kernel).  One lane per pencil when a source has at
        // least 32 Ki pencils (the chunked form's carries and shuffles then
        // cost more than the extra lanes give: 256x256 forward and adjoint
        // run side by side 14 % faster on one lane than on two); else the
        // smallest of 2, 4, 8 that gives one source 64 Ki lanes, with chunks
        // of at least 12 levels.  It depends on the grid only, so a source's
        // arithmetic does not depend on the batch around it.
        // SPARC_STAGE_LANES forces 1, 2, 4 or 8 (a switch the tests use to
        // compare the chunkings)
        if (!c->f32 && (p->option == 4 || p->option == 17)) {
            int q = 1;
            for (int cand = 2; cand <= 8 && c->M < 32768 && (long long)c->M * q < 65536; cand *= 2) {
                const int ch = (c->nz + cand - 1) / cand;
                if (ch < 12 || (cand - 1) * ch >= c->nz) break;
                q = cand;
            }
            if (const char* e = getenv("SPARC_STAGE_LANES")) {
                const int v = atoi(e);
                const int ch = v > 0 ? (c->nz + v - 1) / v : 0;
                if ((v == 1 || v == 2 || v == 4 || v == 8) && (v == 1 || (ch >= 2 && (v - 1) * ch < c->nz))) q = v;
            }
            c->stage_q = q;
            c->stage_chunk = (c->nz + q - 1) / q;
        }
        if ((rc = dalloc(c, &c->zc, (size_t)4 * c->nz * es))) return bail(rc);
        const long long cols = (long long)c->M * S * c->stage_q;
        c->stage_block = 128;
        while (c->stage_block > 32 && (cols + c->stage_block - 1) / c->stage_block < 2LL * nsm) c->stage_block /= 2;
    }
    if (c->f32) {
        // the fused step covers the quiet displacement forms (options 4, 17)
        c->use_fused = fused_supported(c->nz) && (p->option == 4 || p->option == 17) &&
                       getenv("SPARC_FP32_PER_STAGE") == nullptr &&
                       fused_lookback_ok(c->nz, p->option == 4 ? 1 : 3, p->option == 4 ? 0 : 2);
        // modes per CTA of the fused step before any autotuning: 8 (one
        // 512-thread CTA per SM) when it fits and the grid still gives every SM
        // two CTAs, else 4; SPARC_FUSED_MODES forces a shape (a switch the tests
        // use to compare the variants)
        {
            int dev = 0, nsm = 152;
            if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
            cudaGetLastError();
            const long long ctas8 = (long long)((c->M + 7) / 8) * S;
            c->fused_pencils = (fused_fits(8, c->nz, c->nzpml) && ctas8 >= 2LL * nsm) ? 8 : 4;
        }
        if (const char* e = getenv("SPARC_FUSED_MODES")) {
            const int v = atoi(e);
            if (v == 2 || v == 4 || (v == 8 && fused_fits(8, c->nz, c->nzpml))) c->fused_pencils = v;
        }
        // SPARC_TEST_FUSED_NO_TABLE_COPY: the fused step issues no z-table
        // copy, so its bounded wait runs out with nothing in flight (a switch
        // the tests use to exercise the timeout path)
        c->fused_test_nocopy = getenv("SPARC_TEST_FUSED_NO_TABLE_COPY") != nullptr;
        if (c->use_fused &&
            (rc = dalloc(c, (void**)&c->ftab, (size_t)FZ_COUNT * fused_nzp(c->nz) * 4))) return bail(rc);
        if ((rc = dalloc(c, (void**)&c->zt64, (size_t)ZT_COUNT * c->nz * 8))) return bail(rc);
        if ((rc = dalloc(c, (void**)&c->pt64, (size_t)PT_COUNT * c->M * 8))) return bail(rc);
    } else {
        c->zt64 = (double*)c->zt;
        c->pt64 = (double*)c->pt;
    }
    // twiddle tables: n FP64 values, then the same n values in FP32
    if ((rc = dalloc(c, (void**)&c->tw_x, (size_t)p->nx * 12))) return bail(rc);
    if ((rc = dalloc(c, (void**)&c->tw_y, (size_t)std::max(p->ny, 2) * 12))) return bail(rc);
    if ((rc = dalloc(c, &c->tmp, (size_t)c->fs * cs))) return bail(rc);
    if ((rc = dalloc(c, &c->phys, (size_t)c->N * es))) return bail(rc);
    if ((rc = dalloc(c, (void**)&c->phys64, (size_t)c->N * 8))) return bail(rc);
    if ((rc = dalloc(c, (void**)&c->d_flag, 16))) return bail(rc);
    if ((rc = dalloc(c, (void**)&c->d_t0, (size_t)c->S * sizeof(int)))) return bail(rc);
    if ((rc = dalloc(c, (void**)&c->d_time, sizeof(int)))) return bail(rc);
    launch_set_time(c->d_time, 0, c->stream);
    c->t0.assign(c->S, 0);
    c->active_n = c->S;
    c->use_graphs = getenv("SPARC_NO_GRAPHS") == nullptr && !mhd_form;
    if (c->use_fused) {
        fused_prepare(c->nz, c->nzpml);
        if ((rc = dalloc(c, &c->src_plane, (size_t)c->S * c->M * 8))) return bail(rc);
    }
    if (mhd_form && (rc = mhd_create(c))) return bail(rc);
    // twiddles cos/sin(2 pi q / n), q < n/2, exact pi; the FP32 copy (rounded
    // from FP64) follows the FP64 table in the same allocation
    for (int dir = 0; dir < 2; ++dir) {
        int n = dir == 0 ? p->nx : p->ny;
        if (n < 2) continue;
        std::vector<double> tw(n);
        std::vector<float> tw32(n);
        for (int q = 0; q < n / 2; ++q) {
            double ang = 2.0 * M_PI * (double)q / (double)n;
            tw[2 * q] = std::cos(ang);
            tw[2 * q + 1] = std::sin(ang);
        }
        for (int q = 0; q < n; ++q) tw32[q] = (float)tw[q];
        double* dst = dir == 0 ? c->tw_x : c->tw_y;
        if ((rc = upload(c, dst, tw.data(), n * 8)) || (rc = upload(c, dst + n, tw32.data(), n * 4))) return bail(rc);
    }
    c->src_set.assign(c->S, 0);
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) return bail(SPARC_ECUDA);
    *out = c;
    return SPARC_OK;
}

void sparc_gpu_destroy(sparc_ctx* c) {
    if (!c) return;
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (void* p : c->allocs) cudaFree(p);
    if (c->ev_done) cudaEventDestroy(c->ev_done);
    for (cudaEvent_t e : c->slot_ev) cudaEventDestroy(e);
    for (auto& g : c->graphs) cudaGraphExecDestroy(g.exec);
    if (c->mhd) mhd_destroy(c);
    if (c->stream) cudaStreamDestroy(c->stream);
    cudaGetLastError();
    delete c;
}

void* sparc_gpu_stream(sparc_ctx* c) { return c ? (void*)c->stream : nullptr; }
long long sparc_gpu_launch_count(const sparc_ctx* c) { return c ? c->launches : 0; }
long long sparc_gpu_device_bytes(const sparc_ctx* c) { return c ? c->dev_bytes : 0; }

// ---------------------------------------------------------------------------
// set-up: solar_data, stretch, mp_Initialize_RHS(_2d), INIT_DAMPING(_2D), INITIALIZE_STEP
// ---------------------------------------------------------------------------
int sparc_gpu_set_background(sparc_ctx* c, const double* zin, const double* cin, const double* rhoin,
                             const double* pin, const double* gin, const double* gamin) {
    if (!c) return SPARC_EINVAL;
    if (!zin || !cin || !rhoin || !pin || !gin || !gamin) return fail(c, SPARC_EINVAL, "null background array");
    const sparc_params& P = c->P;
    const int nz = c->nz, nx = P.nx, ny = P.ny;
    const bool two_d = (P.option == 17 || P.option == 18);
    for (int k = 0; k < nz; ++k) {
        if (!std::isfinite(zin[k]) || !(cin[k] > 0) || !(rhoin[k] > 0) || !std::isfinite(pin[k]) || !std::isfinite(gin[k]))
            return fail(c, SPARC_EINVAL, "background row " + std::to_string(k + 1) + " is not finite/positive");
        if (k > 0 && !(zin[k] > zin[k - 1])) return fail(c, SPARC_EINVAL, "z must increase with row index");
    }
    c->pi = R4(3.14159265358979);            // initialize.f90:38 (REAL*4 literal)
    c->rsun = R4(69598946770.0);
    c->normx = 1.0 / (double)nx;
    c->normy = 1.0 / (double)ny;
    c->dimc = R4(1.0e6);                       // initialize.f90:751
    c->dimrho = (double)1.0e-3f;               // initialize.f90:755
    c->diml = c->rsun;
    c->stretchx = c->rsun / R4(P.xlength);     // initialize.f90:223-224
    c->stretchy = c->rsun / R4(P.ylength);
    std::vector<double> z(zin, zin + nz), c2(nz), rho0(nz), p0(nz), g(nz), graw(nz);
    for (int k = 0; k < nz; ++k) {             // initialize.f90:759-769
        c2[k] = (cin[k] / c->dimc) * (cin[k] / c->dimc);
        rho0[k] = rhoin[k] / c->dimrho;
        p0[k] = pin[k] / (c->dimrho * (c->dimc * c->dimc));
        g[k] = gin[k] * c->diml / (c->dimc * c->dimc);
        graw[k] = g[k];
    }
    c->zq = z;
    c->cq.resize(nz); c->rhoq.resize(nz);
    for (int k = 0; k < nz; ++k) { c->cq[k] = cin[k] / c->dimc; c->rhoq[k] = rhoin[k] / c->dimrho; }
    compact_coeffs(nz, c->cc64);
    Tri tri[4] = {tri_for(nz, 0), tri_for(nz, 1), tri_for(nz, 2), tri_for(nz, 3)};
    std::vector<double> unstretch, stretch(nz);
    host_dbyd2(z, unstretch, 1, c->cc64, tri[1]);          // initialize.f90:464
    for (int k = 0; k < nz; ++k) stretch[k] = 1.0 / unstretch[k];
    c->deltat = P.timestep * c->dimc / c->diml;               // initialize.f90:472
    // READ_PARAMETERS (initialize.f90:978-981), driver.f90:269-281
    double ts = R4(P.timestep), cad = R4(P.cadforcing);
    c->cadforcing_step = (int)std::floor(cad / ts);
    c->maxtime = (int)std::floor((R4(P.solartime) * 3600.0 + 2.0 / R4(P.nupeak)) / ts) + 2;
    c->maxtime = c->cadforcing_step * (c->maxtime / c->cadforcing_step);
    c->forcing_length = c->maxtime / c->cadforcing_step + 1;
    c->steps = (int)std::floor(R4(P.outputcad) / ts);
    c->freq_filtering = (int)std::floor(60.0 / ts);
    c->num_steps = (int)std::floor((double)c->maxtime * ts / cad) + 2;
    c->num_steps = 2 * (c->num_steps / 2) + 2;
    if (c->steps < 1 || c->freq_filtering < 1 || c->cadforcing_step < 1)
        return fail(c, SPARC_EINVAL, "timestep too large for the output/forcing cadences");
    // e_rad / o_rad (physics.f90:44-63; physics2d.f90:34-54)
    {
        double temp2 = 1.0 + R4(P.excitdep) / c->rsun, temp = 1.0;
        for (int k = 0; k < nz; ++k)
            if (std::fabs(z[k] - temp2) <= temp) { temp = std::fabs(z[k] - temp2); c->e_rad = k + 1; }
        double temp_r = 1.0 + R4(P.obsheight) / c->rsun;
        temp = 1.0;
        for (int k = 0; k < nz; ++k)
            if (std::fabs(z[k] - temp_r) <= temp) { temp = std::fabs(z[k] - temp_r); c->o_rad = k + 1; }
        if (two_d) { c->e_rad = nz - 5; c->o_rad = nz - 1; }
    }
    int ksrc = P.src_k > 0 ? P.src_k : (P.compute_adjoint ? c->o_rad : c->e_rad);
    if (ksrc < 2 || ksrc > nz - 1) return fail(c, SPARC_EINVAL, "source plane must lie strictly inside the box");
    if (P.compute_adjoint) c->delta_width = 2.0 / (z[c->o_rad] - z[c->o_rad - 2]);
    if (P.compute_forward) c->delta_width = 2.0 / (z[c->e_rad] - z[c->e_rad - 2]);
    if (P.src_k > 0) c->delta_width = 2.0 / (z[ksrc] - z[ksrc - 2]);
    // background gradients (physics.f90:204-208)
    std::vector<double> rhoinv(nz), c2rho0(nz), gradrho0, gradp0;
    for (int k = 0; k < nz; ++k) { rhoinv[k] = 1.0 / rho0[k]; c2rho0[k] = c2[k] * rho0[k]; }
    host_dbyd2(rho0, gradrho0, 1, c->cc64, tri[1]);
    host_dbyd2(p0, gradp0, 1, c->cc64, tri[1]);
    for (int k = 0; k < nz; ++k) { gradrho0[k] *= stretch[k]; gradp0[k] *= stretch[k]; }
    // PML profiles (physics.f90:255-303; physics2d.f90:293-342)
    std::vector<double> az(nz), bz(nz);
    {
        int nb = P.npmlbot, nt = P.npmltop;
        double fac_bot = two_d ? 3.0 * 3.0 : 2.0 * 3.0 * 3.0;
        for (int k = 1; k <= nz; ++k) {
            double alphaz = c->pi * R4(0.005) * c->diml / c->dimc, dampz = 0.0;
            if (k < nb + 1) {
                alphaz = c->pi * R4(0.005) * c->diml / c->dimc * (z[k - 1] - z[0]) / (z[nb - 1] - z[0]);
                double tempin = std::sqrt(c2[0]);
                double r = (z[nb - 1] - z[k - 1]) / (z[nb - 1] - z[0]);
                dampz = fac_bot * tempin / (z[nb - 1] - z[0]) * (r * r);
                double fdec = alphaz / (dampz + alphaz);
                gradp0[k - 1] *= fdec;
                gradrho0[k - 1] *= fdec;
                g[k - 1] *= fdec;
            }
            if (k > nz - nt) {
                alphaz = c->pi * R4(0.005) * c->diml / c->dimc * (z[nz - 1] - z[k - 1]) / (z[nz - 1] - z[nz - nt]);
                double tempin = std::sqrt(c2[two_d ? nz - 6 : nz - 1]);
                double r = (z[nz - nt] - z[k - 1]) / (z[nz - 1] - z[nz - nt]);
                dampz = 3.0 * 3.0 * tempin / (z[nz - 1] - z[nz - nt]) * (r * r);
                double fdec = alphaz / (dampz + alphaz);
                gradp0[k - 1] *= fdec;
                gradrho0[k - 1] *= fdec;
                g[k - 1] *= fdec;
            }
            bz[k - 1] = -alphaz - dampz;
            az[k - 1] = -dampz;
        }
    }
    // LDDRK coefficients (step.f90:28-40), REAL*4 optimals
    {
        double opt3 = R4(0.1665579725791151184), opt4 = R4(0.03950410250586729987), opt5 = R4(0.007810706393337838236);
        double b5 = 0.5, b4 = opt3 / b5, b3 = opt4 / (b5 * b4), b2 = opt5 / (b5 * b4 * b3);
        c->betas[0] = 0.0;
        c->betas[1] = b2 * c->deltat;
        c->betas[2] = b3 * c->deltat;
        c->betas[3] = b4 * c->deltat;
        c->betas[4] = b5 * c->deltat;
    }
    // z table
    c->zt_host.assign((size_t)ZT_COUNT * nz, 0.0);
    auto ZR = [&](int row) { return &c->zt_host[(size_t)row * nz]; };
    for (int k = 0; k < nz; ++k) {
        ZR(ZT_STRETCH)[k] = stretch[k];
        ZR(ZT_UNSTRETCH)[k] = unstretch[k];
        ZR(ZT_C2RHO0)[k] = c2rho0[k];
        ZR(ZT_GRADP0)[k] = gradp0[k];
        ZR(ZT_RHO0)[k] = rho0[k];
        ZR(ZT_GRADRHO0)[k] = gradrho0[k];
        ZR(ZT_RHOINV)[k] = rhoinv[k];
        ZR(ZT_G)[k] = g[k];
        ZR(ZT_AZ)[k] = az[k];
        ZR(ZT_BZ)[k] = bz[k];
        ZR(ZT_C2)[k] = c2[k];
        ZR(ZT_GRAW)[k] = graw[k];
        // source_dep(k) = exp(-10.0**(7.0)*4.0*(z(k)-z(e_rad))**2.0), the
        // REAL*4 product of the literals times a REAL*8 square (physics.f90:109)
        const double dzs = z[k] - z[c->e_rad - 1];
        ZR(ZT_SRCDEP)[k] = std::exp(-R4(1.0e7 * 4.0) * (dzs * dzs));
        for (int b = 0; b < 4; ++b) {
            ZR(ZT_TH + 3 * b)[k] = tri[b].low[k];
            ZR(ZT_TH + 3 * b + 1)[k] = 1.0 / tri[b].betad[k];
            ZR(ZT_TH + 3 * b + 2)[k] = tri[b].gam[k];
        }
    }
    // pencil table: derivative multipliers, damping rates, horizontal filter
    c->pt_host.assign((size_t)PT_COUNT * c->M, 0.0);
    {
        const int H = c->H;
        double constx = 2.0 * c->pi / R4(P.xlength) * c->rsun;    // damping.f90:21-22
        double consty = 2.0 * c->pi / R4(P.ylength) * c->rsun;
        double expo = (double)2.2f, six = (double)1.0e-6f;
        for (int iky = 0; iky < ny; ++iky) {
            int kys = (iky <= ny / 2) ? iky : iky - ny;             // signed y wavenumber
            int kya = std::abs(kys);
            for (int ikx = 0; ikx < H; ++ikx) {
                size_t m = (size_t)iky * H + ikx;
                // eyekx (initialize.f90:204-210) on the normalised spectrum; the
                // c2r of the reference drops the Nyquist mode of the derivative
                double kxm = (ikx == nx / 2) ? 0.0 : (double)ikx * c->normx * 2.0 * c->pi * (double)nx * c->stretchx;
                double kym = 0.0;
                if (ny > 1 && iky != ny / 2) kym = (double)kys * c->normy * 2.0 * c->pi * (double)ny * c->stretchy;
                double jj = two_d ? 0.0 : (double)kya;
                double ii = (double)ikx;
                double kay = std::sqrt(constx * constx * (ii * ii) + consty * consty * (jj * jj));
                double gam = c->diml / c->dimc * six * 150.0 * std::pow(kay / 902.0, expo);   // damping.f90:38
                float fx = 1.0f / (1.0f + std::exp(((float)(ikx + 1) - (float)nx / 3.0f) * 1.0f));
                double hf = (double)fx;
                if (!two_d) {
                    float fy = 1.0f / (1.0f + std::exp(((float)(kya + 1) - (float)ny / 3.0f) * 1.0f));
                    hf = hf * (double)fy;
                }
                c->pt_host[PT_KX * (size_t)c->M + m] = kxm;
                c->pt_host[PT_KY * (size_t)c->M + m] = kym;
                // the quiet 2-D form does not damp; the 2-D MHD form does (physics2d.f90:897)
                c->pt_host[PT_DAMP * (size_t)c->M + m] = P.damp_waves && P.option != 17 ? gam : 0.0;
                c->pt_host[PT_HF * (size_t)c->M + m] = hf;
            }
        }
    }
    int rc;
    if (c->f32) {
        if (c->use_fused) {
            // z table of the fused FP32 step, built in FP64 and rounded once:
            // profile rows (with the buoyancy products g rho0/rho0 and
            // g drho0/dz / rho0 folded), and the LU
            // elimination multipliers of the xi_z and p' boundary codes with
            // their chunk products (chunks of FUSED_CH levels; padding rows
            // up to NZP carry zero multipliers)
            const int NZP = fused_nzp(nz);
            const bool d3 = (P.option == 4);
            std::vector<float> ft((size_t)FZ_COUNT * NZP, 0.f);
            auto put = [&](int row, int j, double v) { ft[(size_t)row * NZP + j] = (float)v; };
            for (int j = 0; j < nz; ++j) {
                const double ri = ZR(ZT_RHOINV)[j], g = ZR(ZT_G)[j];
                put(FZ_AZR, j, ZR(ZT_AZ)[j] / ri);   // a_z of psi_p times rho0, the scale of the p' solve undone
                put(FZ_C2R, j, ZR(ZT_C2RHO0)[j]);
                put(FZ_GP, j, ZR(ZT_GRADP0)[j]);
                put(FZ_RI, j, ri);
                put(FZ_E1, j, g * ri * ZR(ZT_RHO0)[j]);
                put(FZ_E2, j, g * ri * ZR(ZT_GRADRHO0)[j]);
                put(FZ_AZ, j, ZR(ZT_AZ)[j]);
                put(FZ_BZ, j, ZR(ZT_BZ)[j]);
            }
            const int bcs[2] = {d3 ? 1 : 3, d3 ? 0 : 2};
            const int base[2] = {FZ_SX, FZ_SP};
            const int lbase[2] = {FZ_LX, FZ_LP};
            const int tp = NZP / FUSED_CH;
            for (int k = 0; k < 2; ++k) {
                std::vector<double> sig(NZP, 1.0);
                for (int j = 0; j < nz; ++j) sig[j] = ZR(ZT_STRETCH)[j] * (k == 1 ? ZR(ZT_RHOINV)[j] : 1.0);
                const FusedRows fr = fused_rows_scaled(fused_rows(nz, NZP, tri[bcs[k]]), sig);
                const std::vector<double> kk = fused_k_row(fr);
                const std::vector<double>* rows[5] = {&fr.ibd, &fr.mm, &kk, &fr.gg, &fr.GG};
                for (int r = 0; r < 5; ++r)
                    for (int j = 0; j < NZP; ++j) put(base[k] + r, j, (*rows[r])[j]);
                std::vector<double> lf, lb;
                fused_lookback(fr, tp, nz, lf, lb);
                for (int i = 0; i < 4 * tp; ++i) {
                    put(lbase[k], i, lf[i]);
                    put(lbase[k] + 1, i, lb[i]);
                }
            }
            if ((rc = upload(c, c->ftab, ft.data(), ft.size() * 4))) return rc;
        }
        std::vector<float> zf(c->zt_host.begin(), c->zt_host.end()), pf(c->pt_host.begin(), c->pt_host.end());
        if ((rc = upload(c, c->zt, zf.data(), zf.size() * 4))) return rc;
        if ((rc = upload(c, c->pt, pf.data(), pf.size() * 4))) return rc;
        if ((rc = upload(c, c->zt64, c->zt_host.data(), c->zt_host.size() * 8))) return rc;
        if ((rc = upload(c, c->pt64, c->pt_host.data(), c->pt_host.size() * 8))) return rc;
        CK(cudaStreamSynchronize(c->stream));
    } else {
        if ((rc = upload(c, c->zt, c->zt_host.data(), c->zt_host.size() * 8))) return rc;
        if ((rc = upload(c, c->pt, c->pt_host.data(), c->pt_host.size() * 8))) return rc;
        if (c->stage_q > 1) {
            // products of the elimination multipliers over each chunk of
            // stage_chunk levels (stage_chunk_kernel): H(j) from the chunk's
            // first level up to j of m = -low/betad, G(j) from j to the chunk's
            // last level of g = -gam(j+1); xi_z code, then p' code
            const bool d3 = (P.option == 4);
            const int bcs[2] = {d3 ? 1 : 3, d3 ? 0 : 2};
            const int C = c->stage_chunk;
            std::vector<double> zc((size_t)4 * nz, 0.0);
            for (int k = 0; k < 2; ++k) {
                const Tri& t = tri[bcs[k]];
                double* H = zc.data() + (size_t)(2 * k) * nz;
                double* G = zc.data() + (size_t)(2 * k + 1) * nz;
                for (int j0 = 0; j0 < nz; j0 += C) {
                    const int j1 = std::min(j0 + C, nz);
                    double pr = 1.0;
                    for (int j = j0; j < j1; ++j) { pr *= -t.low[j] / t.betad[j]; H[j] = pr; }
                    pr = 1.0;
                    for (int j = j1 - 1; j >= j0; --j) { pr *= (j == nz - 1) ? 0.0 : -t.gam[j + 1]; G[j] = pr; }
                }
            }
            if ((rc = upload(c, c->zc, zc.data(), zc.size() * 8))) return rc;
        }
    }
    size_t cs = csz(c);
    CK(cudaMemsetAsync(c->a, 0, (size_t)c->S * c->nf * c->fs * cs, c->stream));
    CK(cudaMemsetAsync(c->scr, 0, (size_t)c->S * c->nf * c->fs * cs, c->stream));
    CK(cudaMemsetAsync(c->pml, 0, (size_t)c->S * 2 * c->ps * cs, c->stream));
    CK(cudaMemsetAsync(c->scrpml, 0, (size_t)c->S * 2 * c->ps * cs, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    c->time = 0;
    launch_set_time(c->d_time, 0, c->stream);
    c->t0.assign(c->S, 0);
    CK(cudaMemsetAsync(c->d_t0, 0, (size_t)c->S * sizeof(int), c->stream));
    CK(cudaStreamSynchronize(c->stream));
    c->have_bg = true;
    c->epoch++;
    return SPARC_OK;
}

// diagnostic view of the set-up (tests): out[0..] = e_rad, o_rad, delta_width, deltat,
// steps, freq_filtering, maxtime, forcing_length, cadforcing_step, num_steps, betas[5]
static_assert(ZT_COUNT == SPARC_ZTAB_ROWS && PT_COUNT == SPARC_PTAB_ROWS, "table rows of the header");
int sparc_gpu_info(sparc_ctx* c, double* out, double* ztab, double* ptab) {
    if (!c || !c->have_bg) return c ? fail(c, SPARC_ESTATE, "no background") : SPARC_EINVAL;
    if (out) {
        int n = 0;
        out[n++] = c->e_rad; out[n++] = c->o_rad; out[n++] = c->delta_width; out[n++] = c->deltat;
        out[n++] = c->steps; out[n++] = c->freq_filtering; out[n++] = c->maxtime; out[n++] = c->forcing_length;
        out[n++] = c->cadforcing_step; out[n++] = c->num_steps;
        for (int i = 0; i < 5; ++i) out[n++] = c->betas[i];
    }
    if (ztab) std::copy(c->zt_host.begin(), c->zt_host.end(), ztab);
    if (ptab) std::copy(c->pt_host.begin(), c->pt_host.end(), ptab);
    return SPARC_OK;
}

// ---------------------------------------------------------------------------
// physical <-> spectral helpers
// ---------------------------------------------------------------------------
// Host planes into the context's representation: normalised half-spectra,
// or (option 10) the dense physical planes themselves.
// bytes between consecutive planes of a field: a spectral plane, or (option 10) a dense physical one
static size_t plane_bytes(const sparc_ctx* c) { return c->mhd ? (size_t)c->NP * esz(c) : (size_t)c->M * csz(c); }

static int to_spec(sparc_ctx* c, const double* host_field, void* spec_dst, int nplanes) {
    long long n = (long long)c->NP * nplanes;
    if (c->mhd) {
        if (c->f32) {
            // staged through phys64 (nz planes) in chunks: the six PML
            // auxiliaries can hold more planes than one field
            for (int off = 0; off < nplanes; off += c->nz) {
                const long long nc = (long long)c->NP * std::min(c->nz, nplanes - off);
                CK(cudaMemcpyAsync(c->phys64, host_field + (long long)off * c->NP, nc * 8, cudaMemcpyHostToDevice,
                                   c->stream));
                launch_copy_convert<float>((float*)spec_dst + (long long)off * c->NP, c->phys64, nc, c->stream);
                c->launches++;
                CKL();
            }
        } else {
            CK(cudaMemcpyAsync(spec_dst, host_field, n * 8, cudaMemcpyHostToDevice, c->stream));
        }
        return SPARC_OK;
    }
    if (nplanes > c->nz) return fail(c, SPARC_EINVAL, "staging of more planes than phys64 holds");
    CK(cudaMemcpyAsync(c->phys64, host_field, n * 8, cudaMemcpyHostToDevice, c->stream));
    if (c->f32) {
        launch_copy_convert<float>((float*)c->phys, c->phys64, n, c->stream);
        fft_phys_to_spec<float>((const float*)c->phys, CP<float>(spec_dst), CP<float>(c->tmp), c->P.nx, c->P.ny, nplanes,
                                c->tw_x, c->tw_y, c->stream);
        c->launches += 3;
    } else {
        fft_phys_to_spec<double>(c->phys64, CP<double>(spec_dst), CP<double>(c->tmp), c->P.nx, c->P.ny, nplanes,
                                 c->tw_x, c->tw_y, c->stream);
        c->launches += 2;
    }
    CKL();
    return SPARC_OK;
}

// spectral (device, T) -> physical FP64 on device (c->phys64)
static int from_spec_dev(sparc_ctx* c, const void* spec_src, int nplanes) {
    long long n = (long long)c->NP * nplanes;
    if (nplanes > c->nz) return fail(c, SPARC_EINVAL, "staging of more planes than phys64 holds");
    if (c->mhd) {
        if (c->f32) {
            launch_copy_back<float>(c->phys64, (const float*)spec_src, n, c->stream);
            c->launches++;
            CKL();
        } else {
            CK(cudaMemcpyAsync(c->phys64, spec_src, n * 8, cudaMemcpyDeviceToDevice, c->stream));
        }
        return SPARC_OK;
    }
    if (c->f32) {
        fft_spec_to_phys<float>(CP<float>((void*)spec_src), (float*)c->phys, CP<float>(c->tmp), c->P.nx, c->P.ny,
                                nplanes, c->tw_x, c->tw_y, c->stream);
        launch_copy_back<float>(c->phys64, (const float*)c->phys, n, c->stream);
        c->launches += 3;
    } else {
        fft_spec_to_phys<double>(CP<double>((void*)spec_src), c->phys64, CP<double>(c->tmp), c->P.nx, c->P.ny, nplanes,
                                 c->tw_x, c->tw_y, c->stream);
        c->launches += 2;
    }
    CKL();
    return SPARC_OK;
}

static int from_spec(sparc_ctx* c, const void* spec_src, double* host_field, int nplanes) {
    // dense planes (MHD) go through phys64 at most nz planes at a time
    const int chunk = c->mhd ? c->nz : nplanes;
    for (int off = 0; off < nplanes; off += chunk) {
        const int np = std::min(chunk, nplanes - off);
        int rc = from_spec_dev(c, (const char*)spec_src + (size_t)off * plane_bytes(c), np);
        if (rc) return rc;
        CK(cudaMemcpyAsync(host_field + (long long)off * c->NP, c->phys64, (size_t)c->NP * np * 8,
                           cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
    }
    return SPARC_OK;
}

static char* field_ptr(sparc_ctx* c, void* base, int src, int field, long long fstride_elems) {
    return (char*)base + ((long long)src * c->nf + field) * fstride_elems * csz(c);
}

int sparc_gpu_set_state(sparc_ctx* c, int src, const double* a, const double* pml) {
    if (!c) return SPARC_EINVAL;
    if (!c->have_bg) return fail(c, SPARC_ESTATE, "set_background first");
    if (src < 0 || src >= c->S || !a) return fail(c, SPARC_EINVAL, "bad slot or null state");
    for (int f = 0; f < c->nf; ++f) {
        int rc = to_spec(c, a + (long long)f * c->N, field_ptr(c, c->a, src, f, c->fs), c->nz);
        if (rc) return rc;
    }
    if (c->mhd) {
        // six PML auxiliaries of option 10, dense planes
        const size_t pb = (size_t)6 * c->nzpml * c->NP * esz(c);
        char* pbase = (char*)mhd_pml(c) + (size_t)src * pb;
        if (pml && c->nzpml > 0) {
            int rc = to_spec(c, pml, pbase, 6 * c->nzpml);
            if (rc) return rc;
        } else {
            CK(cudaMemsetAsync(pbase, 0, pb, c->stream));
        }
        CK(cudaMemsetAsync((char*)mhd_spml(c) + (size_t)src * pb, 0, pb, c->stream));
    } else {
    char* pbase = (char*)c->pml + (long long)src * 2 * c->ps * csz(c);
    if (pml && c->nzpml > 0) {
        for (int f = 0; f < 2; ++f) {
            int rc = to_spec(c, pml + (long long)f * c->NP * c->nzpml, pbase + f * c->ps * csz(c), c->nzpml);
            if (rc) return rc;
        }
    } else {
        CK(cudaMemsetAsync(pbase, 0, 2 * c->ps * csz(c), c->stream));
    }
    }
    CK(cudaMemsetAsync(field_ptr(c, c->scr, src, 0, c->fs), 0, c->nf * c->fs * csz(c), c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return SPARC_OK;
}

int sparc_gpu_get_state(sparc_ctx* c, int src, double* a, double* pml) {
    if (!c) return SPARC_EINVAL;
    if (!c->have_bg) return fail(c, SPARC_ESTATE, "set_background first");
    if (src < 0 || src >= c->S || !a) return fail(c, SPARC_EINVAL, "bad slot or null buffer");
    for (int f = 0; f < c->nf; ++f) {
        int rc = from_spec(c, field_ptr(c, c->a, src, f, c->fs), a + (long long)f * c->N, c->nz);
        if (rc) return rc;
    }
    if (pml && c->nzpml > 0 && c->mhd) {
        const size_t pb = (size_t)6 * c->nzpml * c->NP * esz(c);
        int rc = from_spec(c, (char*)mhd_pml(c) + (size_t)src * pb, pml, 6 * c->nzpml);
        if (rc) return rc;
    } else if (pml && c->nzpml > 0) {
        char* pbase = (char*)c->pml + (long long)src * 2 * c->ps * csz(c);
        for (int f = 0; f < 2; ++f) {
            int rc = from_spec(c, pbase + f * c->ps * csz(c), pml + (long long)f * c->NP * c->nzpml, c->nzpml);
            if (rc) return rc;
        }
    }
    return SPARC_OK;
}

int sparc_gpu_get_field(sparc_ctx* c, int src, int field, int k, double* host) {
    if (!c) return SPARC_EINVAL;
    if (!c->have_bg) return fail(c, SPARC_ESTATE, "set_background first");
    if (src < 0 || src >= c->S || field < 0 || field >= 2 * c->nf || k < 0 || k > c->nz || !host)
        return fail(c, SPARC_EINVAL, "bad slot, field, plane or buffer");
    void* base = field < c->nf ? c->a : c->scr;
    char* fp = field_ptr(c, base, src, field % c->nf, c->fs);
    if (k > 0) return from_spec(c, fp + (long long)(k - 1) * plane_bytes(c), host, 1);
    return from_spec(c, fp, host, c->nz);
}

// ---------------------------------------------------------------------------
// sources
// ---------------------------------------------------------------------------
int sparc_gpu_set_source(sparc_ctx* c, int src, int mode, const double* planes, int L, const double* series,
                         int nseries) {
    if (!c) return SPARC_EINVAL;
    if (!c->have_bg) return fail(c, SPARC_ESTATE, "set_background first");
    if (src < 0 || src >= c->S) return fail(c, SPARC_EINVAL, "bad source slot");
    if (mode == SPARC_SRC_NONE) {
        c->src_set[src] = 0;
        bool any = false;
        for (int s : c->src_set) any = any || s;
        if (!any) c->src_mode = 0;
        return SPARC_OK;
    }
    if (mode != SPARC_SRC_SERIES && mode != SPARC_SRC_LAGRANGE) return fail(c, SPARC_EINVAL, "bad source mode");
    if (!planes || L < 1) return fail(c, SPARC_EINVAL, "source needs at least one plane");
    if (mode == SPARC_SRC_SERIES && (!series || nseries < 1)) return fail(c, SPARC_EINVAL, "series source needs a series");
    if (mode == SPARC_SRC_SERIES) L = 1;
    if (c->src_mode != 0 && c->src_mode != mode) return fail(c, SPARC_EINVAL, "all slots of a context share one source mode");
    if (c->planes && L > c->src_L) return fail(c, SPARC_EINVAL, "plane count exceeds the first allocation");
    size_t cs = csz(c);
    int rc;
    if (!c->planes) {
        if ((rc = dalloc(c, &c->planes, (size_t)c->S * L * c->M * cs))) return rc;
        c->src_L = L;
        c->epoch++;
    }
    if (mode == SPARC_SRC_SERIES) {
        if (!c->series) {
            if ((rc = dalloc(c, (void**)&c->series, (size_t)c->S * nseries * 8))) return rc;
            c->nseries = nseries;
            c->epoch++;
        }
        if (nseries > c->nseries) return fail(c, SPARC_EINVAL, "series longer than the first allocation");
        std::vector<double> ser(c->nseries, 0.0);
        std::copy(series, series + nseries, ser.begin());
        if ((rc = upload(c, c->series + (long long)src * c->nseries, ser.data(), c->nseries * 8))) return rc;
    }
    const size_t pbytes = plane_bytes(c);
    char* dst = (char*)c->planes + (long long)src * c->src_L * pbytes;
    CK(cudaMemsetAsync(dst, 0, (size_t)c->src_L * pbytes, c->stream));
    // planes are normalised spectra of the physical planes (ny,nx), or the
    // physical planes themselves (option 10)
    for (int l0 = 0; l0 < L; l0 += c->nz) {
        int nl = std::min(c->nz, L - l0);
        if ((rc = to_spec(c, planes + (long long)l0 * c->NP, dst + (long long)l0 * pbytes, nl))) return rc;
    }
    CK(cudaStreamSynchronize(c->stream));
    if (c->src_mode != mode) c->epoch++;      // the step kernels' arguments changed
    c->src_mode = mode;
    c->src_set[src] = 1;
    return SPARC_OK;
}

// ---------------------------------------------------------------------------
// time stepping
// ---------------------------------------------------------------------------
}  // extern "C"

template <typename T>
static void make_args(sparc_ctx* c, StageArgs<T>& A, UpdateArgs<T>& U) {
    const sparc_params& P = c->P;
    memset(&A, 0, sizeof(A));
    A.a = CP<T>(c->a); A.scr = CP<T>(c->scr); A.pml = CP<T>(c->pml); A.scrpml = CP<T>(c->scrpml);
    A.ybuf = CP<T>(c->ybuf); A.pbuf = CP<T>(c->pbuf); A.rbuf = CP<T>(c->rbuf);
    A.zt = (const T*)c->zt; A.pt = (const T*)c->pt;
    A.fs = c->fs; A.ps = c->ps; A.M = c->M; A.nz = c->nz;
    A.npmlbot = P.npmlbot; A.npmltop = P.npmltop; A.option = P.option; A.damp = P.damp_waves && P.option != 17;
    A.block = c->stage_block;
    A.q = c->stage_q; A.chunk = c->stage_chunk; A.zc = (const T*)c->zc;
    A.cc.C1 = (T)c->cc64.C1; A.cc.C2 = (T)c->cc64.C2;
    for (int i = 0; i < 5; ++i) A.cc.Cb[i] = (T)c->cc64.Cb[i];
    for (int i = 0; i < 4; ++i) A.cc.Cf[i] = (T)c->cc64.Cf[i];
    A.cc.alpha2 = (T)c->cc64.alpha2; A.cc.beta1 = (T)c->cc64.beta1; A.cc.cnst = (T)c->cc64.cnst;
    // the velocity form centres its source on e_rad in either direction (pml.f90:49)
    int ksrc = P.src_k > 0 ? P.src_k : (P.compute_adjoint && P.option != 2 ? c->o_rad : c->e_rad);
    A.ksrc = ksrc - 1;
    A.src_scale = (T)(c->delta_width / c->zt_host[ZT_RHO0 * c->nz + ksrc - 1]);
    A.planes = CP<T>(c->planes); A.plane_ss = (long long)c->src_L * c->M; A.L = c->src_L;
    A.src_mode = c->src_mode; A.series = c->series; A.nseries = c->nseries;
    A.clk.t0 = c->d_t0;
    A.clk.time = c->d_time;
    A.clk.freq = c->freq_filtering;
    A.clk.two_d = (P.option == 17 || P.option == 18);
    A.clk.gate = c->forcing_length * c->cadforcing_step;
    A.clk.num_steps = c->num_steps;
    A.clk.ts = R4(P.timestep);
    A.clk.cad = R4(P.cadforcing);
    U.a = A.a; U.scr = A.scr; U.pml = A.pml; U.scrpml = A.scrpml; U.pt = A.pt;
    U.fs = c->fs; U.ps = c->ps; U.M = c->M; U.nz = c->nz; U.nzpml = c->nzpml; U.option = P.option;
    U.dt = (T)c->deltat;
    U.clk = A.clk;
    U.block = c->stage_block;
    U.q = c->stage_q; U.chunk = c->stage_chunk; U.ybuf = CP<T>(c->ybuf);
}

// Enqueue nsteps time steps on the context's stream: per step the fused FP32
// kernel (or five stage launches and the update), the surface record, and
// the advance of the device time.  The source of every slot is evaluated on
// its own clock inside the kernels (series index / LAGRANGE_INTERP / 2-D
// gate), from the device time, so the same sequence is valid at any time.
template <typename T>
static int enqueue_steps(sparc_ctx* c, int nsteps) {
    StageArgs<T> A;
    UpdateArgs<T> U;
    make_args<T>(c, A, U);
    FusedArgs Fz;
    const bool fused = c->use_fused && sizeof(T) == 4;
    if (fused) {
        memset(&Fz, 0, sizeof(Fz));
        Fz.a = (float2*)c->a; Fz.scr = (float2*)c->scr; Fz.pml = (float2*)c->pml;
        Fz.ftab = c->ftab; Fz.pt = (const float*)c->pt;
        Fz.unstr_top = (float)c->zt_host[(size_t)ZT_UNSTRETCH * c->nz + c->nz - 1];
        Fz.fs = c->fs; Fz.ps = c->ps; Fz.M = c->M; Fz.nz = c->nz; Fz.nzpml = c->nzpml;
        Fz.npmlbot = c->P.npmlbot; Fz.npmltop = c->P.npmltop; Fz.option = c->P.option;
        Fz.damp = A.damp; Fz.W = fused_w(c->nz);
        for (int i = 0; i < 5; ++i) Fz.betas[i] = (float)c->betas[i];
        Fz.dt = (float)c->deltat;
        Fz.cc.C1 = (float)c->cc64.C1; Fz.cc.C2 = (float)c->cc64.C2;
        for (int i = 0; i < 5; ++i) Fz.cc.Cb[i] = (float)c->cc64.Cb[i];
        for (int i = 0; i < 4; ++i) Fz.cc.Cf[i] = (float)c->cc64.Cf[i];
        Fz.cc.alpha2 = (float)c->cc64.alpha2; Fz.cc.beta1 = (float)c->cc64.beta1; Fz.cc.cnst = (float)c->cc64.cnst;
        Fz.ksrc = A.ksrc; Fz.src_scale = (float)A.src_scale;
        Fz.planes = (const float2*)c->planes; Fz.plane_ss = A.plane_ss; Fz.L = A.L;
        Fz.src_mode = A.src_mode; Fz.series = A.series; Fz.nseries = A.nseries;
        Fz.clk = A.clk;
        Fz.pencils = c->fused_pencils;
        Fz.err = c->d_flag + 1;
        Fz.no_copy = c->fused_test_nocopy;
        Fz.pf_stride = 1;
        Fz.src_plane = (float2*)c->src_plane;
        Fz.wait_limit = c->fused_test_nocopy ? 64 : (1 << 22);
    }
    for (int it = 0; it < nsteps; ++it) {
        if (fused) {
            Fz.write_scr = (it == nsteps - 1 && c->rhs_out) ? 1 : 0;
            if (Fz.src_mode == 2) {
                launch_source_plane(Fz, c->active_n, c->stream);
                c->launches += 1;
            }
            launch_fused(Fz, c->active_n, c->stream);
            c->launches += 1;
            CKL();
        } else {
            for (int rk = 0; rk < 5; ++rk) {
                A.beta = (T)c->betas[rk];
                A.has_scr = (rk > 0);
                launch_stage<T>(A, c->active_n, c->stream);
            }
            launch_update<T>(U, c->active_n, c->stream);
            c->launches += 6;
            CKL();
        }
        if (c->rec_on) {
            // v_z: field 6 of the displacement forms, field 4 of the velocity form
            launch_record<T>(CP<T>(c->a), CP<T>(c->rec), c->d_t0, c->d_time, c->steps, c->rec_max, c->fs, c->M,
                             c->o_rad - 1, c->P.option == 2 ? 3 : 5, c->active_n, c->stream);
            c->launches++;
            CKL();
        }
        launch_tick(c->d_time, c->stream);
        c->launches++;
        CKL();
    }
    return SPARC_OK;
}

// nsteps steps: replayed from a captured graph when the context allows it,
// captured on first use of this step count (and again after any change of
// kernel arguments); launched directly otherwise.
template <typename T>
static int do_steps(sparc_ctx* c, int nsteps) {
    if (nsteps == 0) return SPARC_OK;
    if (c->mhd) return mhd_steps(c, nsteps);
    // A long call replays one graph of kGraphChunk steps (every kernel reads
    // the clock on the device, so a captured chunk is valid at any time) and
    // a graph of the remainder: capture and instantiation stay bounded.  Each
    // chunk's last step also writes scr; the call's last step is still the
    // last to write it.
    constexpr int kGraphChunk = 64;
    if (c->use_graphs && nsteps > kGraphChunk) {
        for (int i = 0; i < nsteps / kGraphChunk; ++i) {
            const int rc = do_steps<T>(c, kGraphChunk);
            if (rc) return rc;
        }
        return do_steps<T>(c, nsteps % kGraphChunk);
    }
    if (c->use_graphs) {
        sparc_ctx::GraphEntry* ge = nullptr;
        for (auto& g : c->graphs)
            if (g.n == nsteps) { ge = &g; break; }
        if (ge && ge->epoch != c->epoch) {
            cudaGraphExecDestroy(ge->exec);
            c->graphs.erase(c->graphs.begin() + (ge - c->graphs.data()));
            ge = nullptr;
        }
        if (!ge) {
            if (c->graphs.size() >= 8) {             // a few step counts per context
                cudaGraphExecDestroy(c->graphs.front().exec);
                c->graphs.erase(c->graphs.begin());
            }
            const long long l0 = c->launches;
            cudaGraph_t graph = nullptr;
            cudaGraphExec_t exec = nullptr;
            bool ok = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
            int rc = ok ? enqueue_steps<T>(c, nsteps) : SPARC_OK;
            if (ok) ok = cudaStreamEndCapture(c->stream, &graph) == cudaSuccess && rc == SPARC_OK;
            if (ok) ok = cudaGraphInstantiate(&exec, graph, 0) == cudaSuccess;
            if (graph) cudaGraphDestroy(graph);
            const long long nl = c->launches - l0;
            c->launches = l0;
            if (!ok) {
                // no graphs for this context: launch directly from now on
                cudaGetLastError();
                if (exec) cudaGraphExecDestroy(exec);
                c->use_graphs = 0;
            } else {
                c->graphs.push_back({nsteps, c->epoch, exec, nl});
                ge = &c->graphs.back();
            }
        }
        if (ge) {
            CK(cudaGraphLaunch(ge->exec, c->stream));
            c->launches += ge->nlaunch;
            c->time += nsteps;
            return SPARC_OK;
        }
    }
    int rc = enqueue_steps<T>(c, nsteps);
    if (rc) return rc;
    c->time += nsteps;
    return SPARC_OK;
}

extern "C" {

int sparc_gpu_step(sparc_ctx* c, int nsteps) {
    if (!c) return SPARC_EINVAL;
    if (!c->have_bg) return fail(c, SPARC_ESTATE, "set_background first");
    if (nsteps < 0) return fail(c, SPARC_EINVAL, "nsteps < 0");
    return c->f32 ? do_steps<float>(c, nsteps) : do_steps<double>(c, nsteps);
}

int sparc_gpu_set_mhd2d_background(sparc_ctx* c, const double* rho, const double* cs, const double* p,
                                   const double* psi) {
    if (!c) return SPARC_EINVAL;
    if (!c->mhd || c->P.option != 18) return fail(c, SPARC_EINVAL, "the 2-D MHD background belongs to option 18");
    if (!c->have_bg) return fail(c, SPARC_ESTATE, "set_background (the quiet column) first");
    if (!p || !rho || !cs || !psi) return fail(c, SPARC_EINVAL, "null background array");
    return mhd2d_set_background(c, p, rho, cs, psi);
}

int sparc_gpu_set_mhd_background(sparc_ctx* c, const double* rho, const double* cs, const double* p,
                                 const double* bx, const double* by, const double* bz) {
    if (!c) return SPARC_EINVAL;
    if (!c->mhd || (c->P.option != 10 && c->P.option != 8))
        return fail(c, SPARC_EINVAL, "the 3-D MHD background belongs to options 8 and 10");
    if (!c->have_bg) return fail(c, SPARC_ESTATE, "set_background (the quiet column) first");
    if (!rho || !cs || !p || !bx || !by || !bz) return fail(c, SPARC_EINVAL, "null background array");
    return mhd_set_background(c, rho, cs, p, bx, by, bz);
}

int sparc_gpu_autotune(sparc_ctx* c, int steps, int* choice, float* ms_per_step) {
    if (!c) return SPARC_EINVAL;
    if (!c->have_bg) return fail(c, SPARC_ESTATE, "set_background first");
    if (c->mhd) return fail(c, SPARC_EINVAL, "option 10 has no launch variants to tune");
    if (steps < 1) return fail(c, SPARC_EINVAL, "steps < 1");
    const bool fused = c->use_fused && c->f32;
    const int cand[3] = {fused ? 4 : 128, fused ? 2 : 64, fused ? 8 : 32};
    const int ncand = (fused && !fused_fits(8, c->nz, c->nzpml)) ? 2 : 3;
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    float best = 0.f;
    int pick = cand[0];
    for (int ic = 0; ic < ncand; ++ic) {
        const int v = cand[ic];
        if (fused) c->fused_pencils = v; else c->stage_block = v;
        c->epoch++;
        int rc = c->f32 ? do_steps<float>(c, steps) : do_steps<double>(c, steps);   // capture and warm
        if (!rc) {
            CK(cudaEventRecord(e0, c->stream));
            rc = c->f32 ? do_steps<float>(c, steps) : do_steps<double>(c, steps);
            CK(cudaEventRecord(e1, c->stream));
        }
        if (rc) { cudaEventDestroy(e0); cudaEventDestroy(e1); return rc; }
        CK(cudaEventSynchronize(e1));
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, e0, e1));
        ms /= steps;
        if (v == cand[0] || ms < best) { best = ms; pick = v; }
    }
    if (fused) c->fused_pencils = pick; else c->stage_block = pick;
    c->epoch++;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (choice) *choice = pick;
    if (ms_per_step) *ms_per_step = best;
    return SPARC_OK;
}

}  // extern "C"

template <typename T>
static int stage_only(sparc_ctx* c, int rk) {
    StageArgs<T> A;
    UpdateArgs<T> U;
    make_args<T>(c, A, U);
    A.beta = (T)c->betas[rk - 1];
    A.has_scr = (rk > 1);
    launch_stage<T>(A, c->active_n, c->stream);
    c->launches++;
    CKL();
    return SPARC_OK;
}

extern "C" {

int sparc_gpu_stage(sparc_ctx* c, int rk) {
    if (!c) return SPARC_EINVAL;
    if (!c->have_bg) return fail(c, SPARC_ESTATE, "set_background first");
    if (rk < 1 || rk > 5) return fail(c, SPARC_EINVAL, "rk must be 1..5");
    return c->f32 ? stage_only<float>(c, rk) : stage_only<double>(c, rk);
}

int sparc_gpu_get_time(const sparc_ctx* c, int* t) {
    if (!c || !t) return SPARC_EINVAL;
    *t = c->time;
    return SPARC_OK;
}
int sparc_gpu_set_time(sparc_ctx* c, int t) {
    if (!c || t < 0) return SPARC_EINVAL;
    c->time = t;
    launch_set_time(c->d_time, t, c->stream);
    CKL();
    return SPARC_OK;
}

int sparc_gpu_sync(sparc_ctx* c, int check_finite) {
    if (!c) return SPARC_EINVAL;
    CK(cudaStreamSynchronize(c->stream));
    if (c->use_fused && c->f32) {
        // a bounded device wait of the fused step that gave up (the z-table bulk copy)
        int tflag = 0;
        CK(cudaMemcpy(&tflag, c->d_flag + 1, 4, cudaMemcpyDeviceToHost));
        if (tflag) {
            CK(cudaMemset(c->d_flag + 1, 0, 4));
            return fail(c, SPARC_ETIMEDOUT, "fused step: the bounded wait for the z-table bulk copy gave up");
        }
    }
    if (check_finite && c->have_bg) {
        CK(cudaMemsetAsync(c->d_flag, 0, 4, c->stream));
        long long n = (long long)c->S * c->nf * c->fs * 2;
        if (c->f32) launch_check_finite_f32((const float*)c->a, n, c->d_flag, c->stream);
        else launch_check_finite_f64((const double*)c->a, n, c->d_flag, c->stream);
        c->launches++;
        int flag = 0;
        CK(cudaMemcpyAsync(&flag, c->d_flag, 4, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        if (flag) return fail(c, SPARC_ENAN, "non-finite value in the state");
    }
    return SPARC_OK;
}

// ---------------------------------------------------------------------------
// surface records
// ---------------------------------------------------------------------------
int sparc_gpu_record_surface(sparc_ctx* c, int enable, int max_records) {
    if (!c) return SPARC_EINVAL;
    c->epoch++;
    if (!enable) { c->rec_on = 0; return SPARC_OK; }
    if (max_records < 1) return fail(c, SPARC_EINVAL, "max_records < 1");
    if (!c->rec || max_records > c->rec_max) {
        if (c->rec) return fail(c, SPARC_EINVAL, "record buffer already allocated smaller");
        int rc = dalloc(c, &c->rec, (size_t)c->S * max_records * c->M * csz(c));
        if (rc) return rc;
        c->rec_max = max_records;
    }
    CK(cudaMemsetAsync(c->rec, 0, (size_t)c->S * c->rec_max * c->M * csz(c), c->stream));
    c->rec_on = 1;
    return SPARC_OK;
}

// records written so far for a slot: outputs at slot times 0, steps, 2*steps, ... < slot time
static int slot_nrec(const sparc_ctx* c, int src) {
    const int lt = c->time - c->t0[src];
    if (lt <= 0 || !c->rec) return 0;
    return std::min(c->rec_max, (lt - 1) / c->steps + 1);
}

int sparc_gpu_get_records(sparc_ctx* c, int src, double* host, int* nrec) {
    if (!c || !nrec) return SPARC_EINVAL;
    if (src < 0 || src >= c->S) return fail(c, SPARC_EINVAL, "bad slot");
    const int n_rec = slot_nrec(c, src);
    *nrec = n_rec;
    if (!host || n_rec == 0) return SPARC_OK;
    const char* base = (const char*)c->rec + (size_t)src * c->rec_max * c->M * csz(c);
    for (int r0 = 0; r0 < n_rec; r0 += c->nz) {
        int n = std::min(c->nz, n_rec - r0);
        int rc = from_spec(c, base + (size_t)r0 * plane_bytes(c), host + (size_t)r0 * c->NP, n);
        if (rc) return rc;
    }
    return SPARC_OK;
}

// ---------------------------------------------------------------------------
// continuous batching: per-slot clocks and the active-slot bound
// ---------------------------------------------------------------------------
int sparc_gpu_slot_reset(sparc_ctx* c, int src) {
    if (!c) return SPARC_EINVAL;
    if (!c->have_bg) return fail(c, SPARC_ESTATE, "set_background first");
    if (src < 0 || src >= c->S) return fail(c, SPARC_EINVAL, "bad slot");
    const size_t cs = csz(c);
    CK(cudaMemsetAsync(field_ptr(c, c->a, src, 0, c->fs), 0, c->nf * c->fs * cs, c->stream));
    CK(cudaMemsetAsync(field_ptr(c, c->scr, src, 0, c->fs), 0, c->nf * c->fs * cs, c->stream));
    CK(cudaMemsetAsync((char*)c->pml + (size_t)src * 2 * c->ps * cs, 0, 2 * c->ps * cs, c->stream));
    CK(cudaMemsetAsync((char*)c->scrpml + (size_t)src * 2 * c->ps * cs, 0, 2 * c->ps * cs, c->stream));
    if (c->mhd) {
        const size_t pb = (size_t)6 * c->nzpml * c->NP * esz(c);
        CK(cudaMemsetAsync((char*)mhd_pml(c) + (size_t)src * pb, 0, pb, c->stream));
        CK(cudaMemsetAsync((char*)mhd_spml(c) + (size_t)src * pb, 0, pb, c->stream));
    }
    if (c->rec) CK(cudaMemsetAsync((char*)c->rec + (size_t)src * c->rec_max * c->M * cs, 0, (size_t)c->rec_max * c->M * cs, c->stream));
    c->t0[src] = c->time;
    CK(cudaMemcpyAsync(c->d_t0 + src, &c->t0[src], sizeof(int), cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return SPARC_OK;
}

int sparc_gpu_slot_time(const sparc_ctx* c, int src, int* local_time) {
    if (!c || !local_time || src < 0 || src >= c->S) return SPARC_EINVAL;
    *local_time = c->time - c->t0[src];
    return SPARC_OK;
}

int sparc_gpu_set_stream_priority(sparc_ctx* c, int level) {
    if (!c) return SPARC_EINVAL;
    if (level < 0) return fail(c, SPARC_EINVAL, "priority level < 0");
    int least = 0, greatest = 0;
    CK(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    const int pr = std::max(greatest, least - level);     // CUDA: numerically lower is more urgent
    CK(cudaStreamSynchronize(c->stream));
    cudaStream_t ns = nullptr;
    CK(cudaStreamCreateWithPriority(&ns, cudaStreamNonBlocking, pr));
    cudaStreamDestroy(c->stream);
    c->stream = ns;
    c->epoch++;                         // step graphs are captured again on first use
    if (c->mhd) return mhd_set_stream_priority(c, pr);
    return SPARC_OK;
}

int sparc_gpu_query(sparc_ctx* c, int* busy) {
    if (!c || !busy) return SPARC_EINVAL;
    const cudaError_t e = cudaStreamQuery(c->stream);
    if (e == cudaSuccess) { *busy = 0; return SPARC_OK; }
    if (e == cudaErrorNotReady) {
        cudaGetLastError();            // not an error: the stream still has work
        *busy = 1;
        return SPARC_OK;
    }
    return fail(c, SPARC_ECUDA, std::string("cudaStreamQuery: ") + cudaGetErrorString(e));
}

int sparc_gpu_set_rhs_output(sparc_ctx* c, int on) {
    if (!c) return SPARC_EINVAL;
    const int v = on ? 1 : 0;
    if (c->rhs_out != v) c->epoch++;    // the flag is an argument of the captured step kernels
    c->rhs_out = v;
    return SPARC_OK;
}

int sparc_gpu_set_active(sparc_ctx* c, int nactive) {
    if (!c) return SPARC_EINVAL;
    if (nactive < 1 || nactive > c->S) return fail(c, SPARC_EINVAL, "nactive out of range");
    if (c->active_n != nactive) c->epoch++;
    c->active_n = nactive;
    return SPARC_OK;
}

// ---------------------------------------------------------------------------
// primitives (FP64, via the same transforms and tables)
// ---------------------------------------------------------------------------
static int ensure_spec64(sparc_ctx* c) {
    if (c->spec64) return SPARC_OK;
    int rc;
    if ((rc = dalloc(c, (void**)&c->spec64, (size_t)c->fs * 16))) return rc;
    if ((rc = dalloc(c, (void**)&c->spec64b, (size_t)c->fs * 16))) return rc;
    if ((rc = dalloc(c, (void**)&c->tmp64, (size_t)c->fs * 16))) return rc;
    return SPARC_OK;
}

static int prim_spectral(sparc_ctx* c, const double* var, double* dvar, int which, int subtract) {
    if (!c) return SPARC_EINVAL;
    if (!c->have_bg) return fail(c, SPARC_ESTATE, "set_background first");
    if (!var || !dvar) return fail(c, SPARC_EINVAL, "null field");
    if (which == 1 && c->P.ny == 1) return fail(c, SPARC_EINVAL, "ddy needs ny > 1");
    int rc = ensure_spec64(c);
    if (rc) return rc;
    CK(cudaMemcpyAsync(c->phys64, var, c->N * 8, cudaMemcpyHostToDevice, c->stream));
    fft_phys_to_spec<double>(c->phys64, c->spec64, c->tmp64, c->P.nx, c->P.ny, c->nz, c->tw_x, c->tw_y, c->stream);
    launch_spec_dxdy<double>(c->spec64b, c->spec64, c->pt64, which, c->M, c->nz, 1, 0, 0, c->stream);
    fft_spec_to_phys<double>(c->spec64b, c->phys64, c->tmp64, c->P.nx, c->P.ny, c->nz, c->tw_x, c->tw_y, c->stream);
    c->launches += 5;
    CKL();
    if (!subtract) {
        CK(cudaMemcpyAsync(dvar, c->phys64, c->N * 8, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
    } else {
        std::vector<double> term(c->N);
        CK(cudaMemcpyAsync(term.data(), c->phys64, c->N * 8, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        for (long long q = 0; q < c->N; ++q) dvar[q] = dvar[q] - term[q];
    }
    return SPARC_OK;
}

int sparc_gpu_ddx(sparc_ctx* c, const double* var, double* dvar) { return prim_spectral(c, var, dvar, 0, 0); }
int sparc_gpu_ddy(sparc_ctx* c, const double* var, double* dvar) { return prim_spectral(c, var, dvar, 1, 0); }
int sparc_gpu_damp(sparc_ctx* c, const double* v, double* rhs) {
    if (c && c->P.option == 17) return fail(c, SPARC_EINVAL, "damping is a 3-D operation");
    return prim_spectral(c, v, rhs, 2, 1);
}

int sparc_gpu_ddz(sparc_ctx* c, const double* var, double* dvar, int bc) {
    if (!c) return SPARC_EINVAL;
    if (!c->have_bg) return fail(c, SPARC_ESTATE, "set_background first");
    if (!var || !dvar || bc < 0 || bc > 3) return fail(c, SPARC_EINVAL, "bad field or bc (0..3)");
    int rc = ensure_spec64(c);
    if (rc) return rc;
    double* din = (double*)c->spec64;     // reuse as two real fields
    double* dout = c->phys64;
    CK(cudaMemcpyAsync(din, var, c->N * 8, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(dout, dvar, c->N * 8, cudaMemcpyHostToDevice, c->stream));
    launch_zderiv_real(c->zt64, c->cc64, din, dout, c->NP, c->nz, bc, c->stream);
    c->launches++;
    CKL();
    CK(cudaMemcpyAsync(dvar, dout, c->N * 8, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return SPARC_OK;
}

// ---------------------------------------------------------------------------
// sensitivity kernels
// ---------------------------------------------------------------------------
}  // extern "C"

// sources per batched snapshot / accumulation pass (bounds the scratch to
// 7 physical + 1 spectral field per source of the group)
static int kernel_group(int S) { return S < 8 ? S : 8; }

// Physical fields of the kernel snapshot of sources s0..s0+G-1 into out
// (field f of source s0+g at out + f*ofs + g*N).  Forward (kernels.f90:
// 197-263): div(xi), f_acc = scr(v) (3), xi (3); adjoint: div(xi), v (3),
// grad(g v_z) (3).  Every pass covers the whole group.
template <typename T>
static int derive_to_phys(sparc_ctx* c, int s0, int G, bool adjoint, T* out, long long ofs) {
    typedef typename CplxOf<T>::type CT;
    const long long fs = c->fs, N = c->N;
    CT* a = CP<T>(c->a) + (long long)s0 * 6 * fs;
    CT* scr = CP<T>(c->scr) + (long long)s0 * 6 * fs;
    CT* D = CP<T>(c->ybuf);      // [G][fs] each
    CT* D2 = CP<T>(c->pbuf);
    CT* D3 = CP<T>(c->rbuf);
    if (!c->gtmp) {
        int rc = dalloc(c, &c->gtmp, (size_t)kernel_group(c->S) * fs * 2 * esz(c));
        if (rc) return rc;
    }
    CT* tmp = CP<T>(c->gtmp);
    Compact<T> cc;
    cc.C1 = (T)c->cc64.C1; cc.C2 = (T)c->cc64.C2;
    for (int i = 0; i < 5; ++i) cc.Cb[i] = (T)c->cc64.Cb[i];
    for (int i = 0; i < 4; ++i) cc.Cf[i] = (T)c->cc64.Cf[i];
    cc.alpha2 = (T)c->cc64.alpha2; cc.beta1 = (T)c->cc64.beta1; cc.cnst = (T)c->cc64.cnst;
    const T* zt = (const T*)c->zt;
    const T* pt = (const T*)c->pt;
    const int nx = c->P.nx, ny = c->P.ny, nz = c->nz, M = c->M;
    const bool use_y = ny > 4;
    // spectral fields of the group -> physical: src_ss = source stride of the
    // input.  One source per transform: its column-pass intermediate (nz
    // planes of the half spectrum, 79 MB in FP32 at 256x256x300) stays in L2
    // for the row pass that reads it right after
    auto tophys = [&](const CT* spec, long long src_ss, T* dst) {
        for (int g = 0; g < G; ++g)
            fft_spec_to_phys_g<T>(spec + (long long)g * src_ss, nz, 0LL, dst + (long long)g * N, tmp, nx, ny, nz,
                                  c->tw_x, c->tw_y, c->stream);
        c->launches += 2 * G;
    };
    // divergence: ddxkern + ddykern + ddzkern(bc=1, filtered)  (COMPUTE_DIV kernels.f90:798-816)
    const int fx = adjoint ? 3 : 0;
    launch_zderiv<T>(zt, cc, a + (fx + 2) * fs, D, M, nz, 1, 1, nullptr, G, 6 * fs, fs, c->stream);
    launch_spec_combine<T>(D, a + fx * fs, use_y ? a + (fx + 1) * fs : nullptr, pt, M, nz, G, fs, 6 * fs, c->stream);
    c->launches += 2;
    tophys(D, fs, out);
    if (!adjoint) {
        for (int q = 0; q < 3; ++q) tophys(scr + (3 + q) * fs, 6 * fs, out + (1 + q) * ofs);   // f_acc
        for (int q = 0; q < 3; ++q) tophys(a + q * fs, 6 * fs, out + (4 + q) * ofs);           // f_xi
    } else {
        for (int q = 0; q < 3; ++q) tophys(a + (3 + q) * fs, 6 * fs, out + (1 + q) * ofs);     // a_v
        // grad(a_vz * grav) (kernels.f90:299-304)
        launch_spec_scale_z<T>(D2, a + 5 * fs, zt, ZT_GRAW, M, nz, G, fs, 6 * fs, c->stream);
        launch_spec_dxdy<T>(D3, D2, pt, 0, M, nz, G, fs, fs, c->stream);
        c->launches += 2;
        tophys(D3, fs, out + 4 * ofs);
        if (use_y) {
            launch_spec_dxdy<T>(D3, D2, pt, 1, M, nz, G, fs, fs, c->stream);
            c->launches++;
            tophys(D3, fs, out + 5 * ofs);
        } else {
            for (int g = 0; g < G; ++g)
                CK(cudaMemsetAsync(out + 5 * ofs + (long long)g * N, 0, N * sizeof(T), c->stream));
        }
        launch_zderiv<T>(zt, cc, D2, D3, M, nz, 1, 1, nullptr, G, fs, fs, c->stream);
        c->launches++;
        tophys(D3, fs, out + 6 * ofs);
    }
    CKL();
    return SPARC_OK;
}

extern "C" {

int sparc_gpu_snapshot(sparc_ctx* c, int snap, int nsnap) {
    if (!c) return SPARC_EINVAL;
    if (!c->have_bg) return fail(c, SPARC_ESTATE, "set_background first");
    if (c->P.option == 2 || (c->mhd && c->P.option != 18))
        return fail(c, SPARC_EINVAL, "sensitivity kernels are built for the displacement forms 4, 17 and 18 "
                                     "(the reference computes kernels in 2-D)");
    if (!c->rhs_out)
        return fail(c, SPARC_ESTATE, "the forward snapshot reads the stage right-hand side (f_acc): "
                                     "sparc_gpu_set_rhs_output(ctx, 1) first");
    if (!c->store) {
        if (nsnap < 1) return fail(c, SPARC_EINVAL, "nsnap < 1");
        int rc = dalloc(c, &c->store, (size_t)nsnap * c->S * 7 * c->N * esz(c));
        if (rc) return rc;
        c->store_n = nsnap;
        c->slot_ev.assign(nsnap, nullptr);
        c->slot_pending.assign(nsnap, 0);
        for (int i = 0; i < nsnap; ++i) CK(cudaEventCreateWithFlags(&c->slot_ev[i], cudaEventDisableTiming));
    }
    if (snap < 0 || snap >= c->store_n) return fail(c, SPARC_EINVAL, "snapshot index out of range");
    if (c->slot_pending[snap]) {           // an adjoint context still reads this slot
        CK(cudaStreamWaitEvent(c->stream, c->slot_ev[snap], 0));
        c->slot_pending[snap] = 0;
    }
    const int G = kernel_group(c->S);
    const long long ofs = (long long)c->S * c->N;          // field stride of the store
    for (int s0 = 0; s0 < c->S; s0 += G) {
        const int g = std::min(G, c->S - s0);
        char* dst = (char*)c->store + ((size_t)snap * 7 * c->S + s0) * c->N * esz(c);
        int rc = c->mhd ? mhd2d_derive(c, s0, g, false, dst, ofs)
                        : (c->f32 ? derive_to_phys<float>(c, s0, g, false, (float*)dst, ofs)
                                  : derive_to_phys<double>(c, s0, g, false, (double*)dst, ofs));
        if (rc) return rc;
    }
    return SPARC_OK;
}

int sparc_gpu_kernel_reset(sparc_ctx* c) {
    if (!c) return SPARC_EINVAL;
    if (!c->kacc) {
        int rc = dalloc(c, (void**)&c->kacc, (size_t)c->S * 3 * c->N * 8);
        if (rc) return rc;
    }
    CK(cudaMemsetAsync(c->kacc, 0, (size_t)c->S * 3 * c->N * 8, c->stream));
    if (c->mhd && c->P.option == 18) return mhd2d_kernel_b_reset(c);
    return SPARC_OK;
}

int sparc_gpu_kernel_accumulate(sparc_ctx* fwd, int snap, sparc_ctx* c) {
    if (!fwd || !c) return SPARC_EINVAL;
    if (!c->have_bg || !fwd->have_bg) return fail(c, SPARC_ESTATE, "set_background first");
    if (!fwd->store || snap < 0 || snap >= fwd->store_n) return fail(c, SPARC_EINVAL, "no such forward snapshot");
    if (fwd->S != c->S || fwd->N != c->N || fwd->f32 != c->f32 || fwd->P.option != c->P.option)
        return fail(c, SPARC_EINVAL, "forward/adjoint contexts differ");
    if (c->mhd && c->P.option != 18) return fail(c, SPARC_EINVAL, "kernels of the 3-D MHD forms are not built");
    if (!c->kacc) { int rc = sparc_gpu_kernel_reset(c); if (rc) return rc; }
    const int G = kernel_group(c->S);
    if (!c->ktemp) { int rc = dalloc(c, &c->ktemp, (size_t)7 * G * c->N * esz(c)); if (rc) return rc; }
    // the forward snapshot is written on the forward context's stream: the
    // adjoint stream waits for it (no host synchronisation)
    CK(cudaEventRecord(fwd->ev_done, fwd->stream));
    CK(cudaStreamWaitEvent(c->stream, fwd->ev_done, 0));
    const long long N = c->N, sfs = (long long)c->S * N;     // store field stride
    for (int s0 = 0; s0 < c->S; s0 += G) {
        const int g = std::min(G, c->S - s0);
        const size_t f7 = ((size_t)snap * 7 * c->S + s0) * N;  // element offset of field 0, source s0
        double* acc = c->kacc + (size_t)s0 * 3 * N;
        int rc;
        const double* c2f = mhd_kernel_c2(c);           // a 2-D MHD background varies in x
        if (c->f32) {
            rc = c->mhd ? mhd2d_derive(c, s0, g, true, c->ktemp, (long long)g * N)
                        : derive_to_phys<float>(c, s0, g, true, (float*)c->ktemp, (long long)g * N);
            if (rc) return rc;
            launch_kernel_accum<float>(acc, (const float*)fwd->store + f7, sfs, (const float*)c->ktemp,
                                       (long long)g * N, c->zt64, c->NP, c->nz, c->P.ny > 4, g, c->stream, c2f);
            if (c->mhd && (rc = mhd2d_kernel_b_accumulate(c, (const float*)fwd->store + f7, sfs, c->ktemp,
                                                          (long long)g * N, s0, g)))
                return rc;
        } else {
            rc = c->mhd ? mhd2d_derive(c, s0, g, true, c->ktemp, (long long)g * N)
                        : derive_to_phys<double>(c, s0, g, true, (double*)c->ktemp, (long long)g * N);
            if (rc) return rc;
            launch_kernel_accum<double>(acc, (const double*)fwd->store + f7, sfs, (const double*)c->ktemp,
                                        (long long)g * N, c->zt64, c->NP, c->nz, c->P.ny > 4, g, c->stream, c2f);
            if (c->mhd && (rc = mhd2d_kernel_b_accumulate(c, (const double*)fwd->store + f7, sfs, c->ktemp,
                                                          (long long)g * N, s0, g)))
                return rc;
        }
        c->launches++;
        CKL();
    }
    // a later snapshot into this slot waits for these reads of it; the
    // forward context's other work does not wait
    CK(cudaEventRecord(fwd->slot_ev[snap], c->stream));
    fwd->slot_pending[snap] = 1;
    return SPARC_OK;
}

// Final scaling of the kernels (kernels.f90:523-539) into the device buffer
// out (3 N doubles), enqueued on the context's stream.
static int kernels_finish(sparc_ctx* c, int src, int sum_slots, double* out) {
    if (!c->kacc) return fail(c, SPARC_ESTATE, "no kernel accumulation yet");
    if (src < 0 || src >= c->S) return fail(c, SPARC_EINVAL, "bad slot");
    int stepskern = c->steps;                         // kernels.f90:190
    double ts = R4(c->P.timestep);
    double dimen = std::pow(c->diml * (double)1.0e-8f, -3.0);            // kernels.f90:523
    if (c->P.ny <= 4) dimen = 1.0 / (c->diml * (double)1.0e-8f * R4(c->P.xlength) * (double)1.0e-8f);
    double sc = stepskern * ts * dimen * 2.0, sr = stepskern * ts * dimen;
    const double* acc = c->kacc + (sum_slots ? 0 : (size_t)src * 3 * c->N);
    launch_kernel_finish(out, acc, c->zt64, c->NP, c->nz, sc, sr, sum_slots ? c->S : 1, 3 * c->N, c->stream,
                         mhd_kernel_rho0(c), mhd_kernel_c2(c));
    c->launches++;
    CKL();
    return SPARC_OK;
}

int sparc_gpu_kernels_device(sparc_ctx* c, int src, int sum_slots, double* dev_out) {
    if (!c) return SPARC_EINVAL;
    if (!dev_out) return fail(c, SPARC_EINVAL, "null output buffer");
    return kernels_finish(c, src, sum_slots, dev_out);
}

int sparc_gpu_kernels(sparc_ctx* c, int src, int sum_slots, double* kc, double* krho, double* hess) {
    if (!c) return SPARC_EINVAL;
    if (!c->kacc) return fail(c, SPARC_ESTATE, "no kernel accumulation yet");
    if (src < 0 || src >= c->S) return fail(c, SPARC_EINVAL, "bad slot");
    double* out = nullptr;
    int rc = dalloc(c, (void**)&out, (size_t)3 * c->N * 8);
    if (rc) return rc;
    if ((rc = kernels_finish(c, src, sum_slots, out))) return rc;
    if (kc) CK(cudaMemcpyAsync(kc, out, c->N * 8, cudaMemcpyDeviceToHost, c->stream));
    if (krho) CK(cudaMemcpyAsync(krho, out + c->N, c->N * 8, cudaMemcpyDeviceToHost, c->stream));
    if (hess) CK(cudaMemcpyAsync(hess, out + 2 * c->N, c->N * 8, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    // release the staging buffer
    cudaFree(out);
    c->allocs.erase(std::remove(c->allocs.begin(), c->allocs.end(), (void*)out), c->allocs.end());
    c->dev_bytes -= (long long)3 * c->N * 8;
    return SPARC_OK;
}

// synth == nullptr: the surface records of slot src on the device.
// adj != nullptr: ADJOINT_SOURCE_FILT (misfit, nmeas: one value);
// adj == nullptr: MISFIT_ALL (misfit, nmeas: [3 bands][3 sets]).
static int adjoint_source(sparc_ctx* c, int src, const double* synth, const double* data, int nt,
                          const sparc_adjsrc_params* ap, int* windows, double* adj, double* misfit, int* nmeas) {
    if (!c) return SPARC_EINVAL;
    if (!c->have_bg) return fail(c, SPARC_ESTATE, "set_background first");
    if (c->P.ny != 1) return fail(c, SPARC_EINVAL, "the adjoint source and misfit are written for 2-D runs (ny = 1)");
    if (src < 0 || src >= c->S || !data || !ap || !windows || !misfit || !nmeas)
        return fail(c, SPARC_EINVAL, "bad slot or null argument");
    if (nt < 1) return fail(c, SPARC_EINVAL, "nt < 1");
    if (!synth && (!c->rec || slot_nrec(c, src) < nt))
        return fail(c, SPARC_ESTATE, "fewer surface records than nt (record_surface and steps first)");
    const long long NP = c->NP;
    double* acc = nullptr;
    int rc = dalloc(c, (void**)&acc, (size_t)nt * NP * 8);
    if (rc) return rc;
    if (synth) {
        if (cudaMemcpyAsync(acc, synth, (size_t)nt * NP * 8, cudaMemcpyHostToDevice, c->stream) != cudaSuccess)
            rc = fail(c, SPARC_ECUDA, "upload of the synthetic");
    } else {
        // the synthetic: records of the slot as FP64 physical planes, on the device
        const char* base = (const char*)c->rec + (size_t)src * c->rec_max * c->M * csz(c);
        for (int r0 = 0; r0 < nt && !rc; r0 += c->nz) {
            const int n = std::min(c->nz, nt - r0);
            rc = from_spec_dev(c, base + (size_t)r0 * plane_bytes(c), n);
            if (!rc && cudaMemcpyAsync(acc + (size_t)r0 * NP, c->phys64, (size_t)n * NP * 8, cudaMemcpyDeviceToDevice,
                                       c->stream) != cudaSuccess)
                rc = fail(c, SPARC_ECUDA, "copy of the records");
        }
    }
    if (!rc) {
        AdjSrcArgs a;
        a.x00 = ap->x00; a.t1 = ap->t1_min; a.dt = ap->dt_min; a.linesearch = ap->linesearch;
        for (int m = 0; m < 3; ++m) {
            a.have_ridge[m] = ap->have_ridge[m];
            for (int q = 0; q < 3; ++q) a.ridge[m][q] = ap->ridge[m][q];
        }
        for (int m = 0; m < 2; ++m) {
            a.have_band[m] = ap->have_band[m];
            for (int q = 0; q < 2; ++q) a.band[m][q] = ap->band[m][q];
        }
        std::string why;
        const int r = adj ? adjsrc_compute(c->stream, acc, data, nt, (int)NP, c->P.xlength, c->P.outputcad, a, windows,
                                           adj, misfit, nmeas, why)
                          : misfit_all_compute(c->stream, acc, data, nt, (int)NP, c->P.xlength, c->P.outputcad, a,
                                               windows, misfit, nmeas, why);
        if (r == 1) rc = fail(c, SPARC_EINVAL, why);
        else if (r == 2) rc = fail(c, SPARC_ECUDA, why);
    }
    cudaFree(acc);
    c->allocs.erase(std::remove(c->allocs.begin(), c->allocs.end(), (void*)acc), c->allocs.end());
    c->dev_bytes -= (long long)nt * NP * 8;
    return rc;
}

int sparc_gpu_adjoint_source(sparc_ctx* c, int src, const double* data, int nt, const sparc_adjsrc_params* ap,
                             int* windows, double* adj, double* misfit, int* nmeas) {
    if (!adj) return c ? fail(c, SPARC_EINVAL, "null adjoint source") : SPARC_EINVAL;
    return adjoint_source(c, src, nullptr, data, nt, ap, windows, adj, misfit, nmeas);
}

int sparc_gpu_misfit_all(sparc_ctx* c, int src, const double* synth, const double* data, int nt,
                         const sparc_adjsrc_params* ap, int* windows, double* misfit, int* nmeas) {
    return adjoint_source(c, src, synth, data, nt, ap, windows, nullptr, misfit, nmeas);
}

int sparc_gpu_adjoint_source_host(sparc_ctx* c, const double* synth, const double* data, int nt,
                                  const sparc_adjsrc_params* ap, int* windows, double* adj, double* misfit,
                                  int* nmeas) {
    if (!synth || !adj) return c ? fail(c, SPARC_EINVAL, "null synthetic or adjoint source") : SPARC_EINVAL;
    return adjoint_source(c, 0, synth, data, nt, ap, windows, adj, misfit, nmeas);
}

int sparc_gpu_kernels_b(sparc_ctx* c, int src, int sum_slots, double* kbx, double* kbz, double* kpsi) {
    if (!c) return SPARC_EINVAL;
    if (!c->mhd || c->P.option != 18) return fail(c, SPARC_EINVAL, "B-field kernels belong to option 18");
    if (src < 0 || src >= c->S) return fail(c, SPARC_EINVAL, "bad slot");
    return mhd2d_kernels_b(c, src, sum_slots, kbx, kbz, kpsi);
}

// ---------------------------------------------------------------------------
// model update of an inversion iteration (grad.py:158-301)
// ---------------------------------------------------------------------------
static int ensure_update(sparc_ctx* c) {
    if (c->upd) return SPARC_OK;
    int rc = ensure_spec64(c);
    if (rc) return rc;
    return dalloc(c, (void**)&c->upd, ((size_t)3 * c->N + c->M + c->nz + kReduceScratch + 8) * 8);
}

// scratch: fields f0, f1, f2 (N each), the filterx multiplier (M), rho_z
// (nz) and the reduction slots
struct UpdBufs { double *f0, *f1, *f2, *mul, *rho, *res, *red; };
static UpdBufs upd_bufs(sparc_ctx* c) {
    UpdBufs b;
    b.f0 = c->upd;
    b.f1 = b.f0 + c->N;
    b.f2 = b.f1 + c->N;
    b.mul = b.f2 + c->N;
    b.rho = b.mul + c->M;
    b.res = b.rho + c->nz;
    b.red = b.res + 8;
    return b;
}

// filterx (grad.py:47-61) of src into dst: the half spectrum along x times
// rfft(exp(-x^2 / 32)), x = fftfreq(nx) nx.  The Gaussian is real and even,
// so its rfft is the real cosine sum; the same factor multiplies every ky.
static int filterx_dev(sparc_ctx* c, const UpdBufs& b, const double* src, double* dst) {
    const int nx = c->P.nx, ny = c->P.ny, H = nx / 2 + 1;
    std::vector<double> g(nx), mul((size_t)c->M);
    for (int i = 0; i < nx; ++i) {
        const double x = (double)(i <= (nx - 1) / 2 ? i : i - nx);
        g[i] = std::exp(-(x * x) / (2.0 * 16.0));
    }
    const double two_pi = 2.0 * std::acos(-1.0);      // numpy's rfft: full FP64 pi, not the context's REAL*4 one
    for (int k = 0; k < H; ++k) {
        double acc = 0.0;
        for (int i = 0; i < nx; ++i) acc += g[i] * std::cos(two_pi * (double)((long long)k * i % nx) / nx);
        for (int y = 0; y < ny; ++y) mul[(size_t)y * H + k] = acc;
    }
    int rc = upload(c, b.mul, mul.data(), mul.size() * 8);
    if (rc) return rc;
    fft_phys_to_spec<double>(src, c->spec64, c->tmp64, nx, ny, c->nz, c->tw_x, c->tw_y, c->stream, b.mul);
    fft_spec_to_phys<double>(c->spec64, dst, c->tmp64, nx, ny, c->nz, c->tw_x, c->tw_y, c->stream);
    CKL();
    // mul is a host vector: the upload must land before it goes out of scope
    CK(cudaStreamSynchronize(c->stream));
    return SPARC_OK;
}

int sparc_gpu_gradient(sparc_ctx* c, const double* kc_sum, const double* kpsi_sum, const double* hess_sum,
                       const double* rho_z, double* grad_c, double* grad_psi) {
    if (!c) return SPARC_EINVAL;
    if (!c->have_bg) return fail(c, SPARC_ESTATE, "set_background first (the transform tables)");
    if (!hess_sum || !rho_z) return fail(c, SPARC_EINVAL, "null hessian or rho_z");
    if ((grad_c && !kc_sum) || (grad_psi && !kpsi_sum)) return fail(c, SPARC_EINVAL, "null kernel for a requested gradient");
    int rc = ensure_update(c);
    if (rc) return rc;
    const UpdBufs b = upd_bufs(c);
    const long long N = c->N, NP = c->NP;
    if ((rc = upload(c, b.f0, hess_sum, N * 8))) return rc;
    if ((rc = upload(c, b.rho, rho_z, (size_t)c->nz * 8))) return rc;
    launch_precondition(b.f0, b.rho, NP, c->nz, b.res, c->stream);
    CKL();
    if (grad_c) {
        if ((rc = upload(c, b.f1, kc_sum, N * 8))) return rc;
        launch_divide(b.f1, b.f1, b.f0, N, c->stream);
        if ((rc = filterx_dev(c, b, b.f1, b.f2))) return rc;
        launch_filterz_smooth(b.f1, b.f2, NP, c->nz, c->stream);
        CKL();
        CK(cudaMemcpyAsync(grad_c, b.f1, N * 8, cudaMemcpyDeviceToHost, c->stream));
    }
    if (grad_psi) {
        if ((rc = upload(c, b.f1, kpsi_sum, N * 8))) return rc;
        launch_divide(b.f1, b.f1, b.f0, N, c->stream);
        if ((rc = filterx_dev(c, b, b.f1, b.f2))) return rc;
        launch_antisymmetrize(b.f1, b.f2, (long long)c->nz * c->P.ny, c->P.nx, c->stream);
        if (!launch_gaussian_z(b.f2, b.f1, NP, c->nz, 2.0, c->stream)) return fail(c, SPARC_EINVAL, "gaussian taps");
        CKL();
        CK(cudaMemcpyAsync(grad_psi, b.f2, N * 8, cudaMemcpyDeviceToHost, c->stream));
    }
    CK(cudaStreamSynchronize(c->stream));
    return SPARC_OK;
}

int sparc_gpu_update_models(sparc_ctx* c, const double* grad_c, const double* grad_psi, const double* last_grad_psi,
                            const double* last_update_c, const double* last_update_psi, const double* model_psi,
                            double eps, int nmodels, double* update_c, double* update_psi, double* test_psi,
                            double* con) {
    if (!c) return SPARC_EINVAL;
    if (!grad_psi) return fail(c, SPARC_EINVAL, "null gradient_vectorpsi");
    const bool cg = last_grad_psi != nullptr;
    if (cg && (!last_update_psi || (update_c && !last_update_c)))
        return fail(c, SPARC_EINVAL, "conjugate gradient needs the last gradient_vectorpsi, update_c and update_vectorpsi");
    if (update_c && !grad_c) return fail(c, SPARC_EINVAL, "update_c requested without gradient_c");
    if (nmodels < 0 || (nmodels > 0 && (!model_psi || !test_psi))) return fail(c, SPARC_EINVAL, "bad test-model request");
    int rc = ensure_update(c);
    if (rc) return rc;
    const UpdBufs b = upd_bufs(c);
    const long long N = c->N;
    double h[3] = {0.0, 0.0, 0.0};
    double cn = 0.0;
    if ((rc = upload(c, b.f0, grad_psi, N * 8))) return rc;
    if (cg) {
        // con = sum g (g - g_last) / sum g_last^2, floored at 0 (grad.py:218-223)
        if ((rc = upload(c, b.f1, last_grad_psi, N * 8))) return rc;
        launch_reduce(b.res, b.f1, nullptr, N, b.red, c->stream);
        launch_sub(b.f1, b.f0, b.f1, N, c->stream);
        launch_reduce(b.res + 4, b.f0, b.f1, N, b.red, c->stream);
        CKL();
        double hr[8];
        CK(cudaMemcpyAsync(hr, b.res, sizeof(hr), cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        cn = hr[4] / hr[0];
        if (cn < 0) cn = 0.0;
        if ((rc = upload(c, b.f1, last_update_psi, N * 8))) return rc;
        launch_axpy_c(b.f0, b.f0, b.f1, cn, N, c->stream);
        CKL();
    }
    if (con) *con = cn;
    if (update_psi) CK(cudaMemcpyAsync(update_psi, b.f0, N * 8, cudaMemcpyDeviceToHost, c->stream));
    if (update_c) {
        if ((rc = upload(c, b.f1, grad_c, N * 8))) return rc;
        if (cg) {
            if ((rc = upload(c, b.f2, last_update_c, N * 8))) return rc;
            launch_axpy_c(b.f1, b.f1, b.f2, cn, N, c->stream);
            CKL();
        }
        CK(cudaMemcpyAsync(update_c, b.f1, N * 8, cudaMemcpyDeviceToHost, c->stream));
    }
    if (nmodels > 0) {
        // test_vectorpsi_i = model + eps i rms(model) u / max|u| (grad.py:282-301)
        if ((rc = upload(c, b.f1, model_psi, N * 8))) return rc;
        launch_reduce(b.res, b.f0, nullptr, N, b.red, c->stream);        // res[1] = max |u|
        launch_reduce(b.res + 4, b.f1, nullptr, N, b.red, c->stream);    // res[4] = sum model^2
        CKL();
        CK(cudaMemcpyAsync(h, b.res + 4, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        const double scale = std::sqrt(h[0] / (double)N);
        for (int i = 1; i <= nmodels; ++i) {
            launch_test_model(b.f2, b.f1, b.f0, b.res, eps * i * scale, N, c->stream);
            CKL();
            CK(cudaMemcpyAsync(test_psi + (size_t)(i - 1) * N, b.f2, N * 8, cudaMemcpyDeviceToHost, c->stream));
        }
    }
    CK(cudaStreamSynchronize(c->stream));
    return SPARC_OK;
}

// ---------------------------------------------------------------------------
// device-resident checkpoints (checkpointed recomputation of the forward run)
// ---------------------------------------------------------------------------
int sparc_gpu_save_device(sparc_ctx* c, int idx, int capacity) {
    if (!c) return SPARC_EINVAL;
    if (c->mhd) return fail(c, SPARC_EINVAL, "checkpoints hold the quiet-Sun state layout (not the MHD forms)");
    if (!c->have_bg) return fail(c, SPARC_ESTATE, "set_background first");
    size_t na = (size_t)c->S * c->nf * c->fs * csz(c), np = (size_t)c->S * 2 * c->ps * csz(c);
    if (!c->dck) {
        if (capacity < 1) return fail(c, SPARC_EINVAL, "capacity < 1");
        int rc = dalloc(c, &c->dck, (size_t)capacity * (na + np));
        if (rc) return rc;
        c->dck_n = capacity;
        c->dck_time.assign(capacity, -1);
    }
    if (idx < 0 || idx >= c->dck_n) return fail(c, SPARC_EINVAL, "device checkpoint index out of range");
    char* dst = (char*)c->dck + (size_t)idx * (na + np);
    CK(cudaMemcpyAsync(dst, c->a, na, cudaMemcpyDeviceToDevice, c->stream));
    CK(cudaMemcpyAsync(dst + na, c->pml, np, cudaMemcpyDeviceToDevice, c->stream));
    c->dck_time[idx] = c->time;
    return SPARC_OK;
}

int sparc_gpu_load_device(sparc_ctx* c, int idx) {
    if (!c) return SPARC_EINVAL;
    if (c->mhd) return fail(c, SPARC_EINVAL, "checkpoints hold the quiet-Sun state layout (not the MHD forms)");
    if (!c->dck || idx < 0 || idx >= c->dck_n || c->dck_time[idx] < 0)
        return fail(c, SPARC_EINVAL, "no such device checkpoint");
    size_t na = (size_t)c->S * c->nf * c->fs * csz(c), np = (size_t)c->S * 2 * c->ps * csz(c);
    const char* src = (const char*)c->dck + (size_t)idx * (na + np);
    CK(cudaMemcpyAsync(c->a, src, na, cudaMemcpyDeviceToDevice, c->stream));
    CK(cudaMemcpyAsync(c->pml, src + na, np, cudaMemcpyDeviceToDevice, c->stream));
    CK(cudaMemsetAsync(c->scr, 0, na, c->stream));
    CK(cudaMemsetAsync(c->scrpml, 0, np, c->stream));
    c->time = c->dck_time[idx];
    launch_set_time(c->d_time, c->time, c->stream);
    return SPARC_OK;
}

// ---------------------------------------------------------------------------
// checkpoint / restore: raw spectral state of every slot + time, FNV-1a checksum
// ---------------------------------------------------------------------------
static uint64_t fnv1a(const unsigned char* p, size_t n, uint64_t h) {
    for (size_t i = 0; i < n; ++i) { h ^= p[i]; h *= 1099511628211ULL; }
    return h;
}

struct CkHeader {
    char magic[8];
    int32_t abi, nx, ny, nz, npmlbot, npmltop, option, precision, nsrc, time;
    uint64_t payload_bytes, checksum;
};

int sparc_gpu_checkpoint(sparc_ctx* c, const char* path) {
    if (!c || !path) return SPARC_EINVAL;
    if (c->mhd) return fail(c, SPARC_EINVAL, "checkpoints hold the quiet-Sun state layout (not the MHD forms)");
    if (!c->have_bg) return fail(c, SPARC_ESTATE, "set_background first");
    size_t na = (size_t)c->S * c->nf * c->fs * csz(c), np = (size_t)c->S * 2 * c->ps * csz(c);
    std::vector<unsigned char> buf(na + np);
    CK(cudaMemcpyAsync(buf.data(), c->a, na, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(buf.data() + na, c->pml, np, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    CkHeader h;
    memset(&h, 0, sizeof(h));
    memcpy(h.magic, "SPARCGPU", 8);
    h.abi = SPARC_GPU_ABI_VERSION; h.nx = c->P.nx; h.ny = c->P.ny; h.nz = c->nz;
    h.npmlbot = c->P.npmlbot; h.npmltop = c->P.npmltop; h.option = c->P.option; h.precision = c->P.precision;
    h.nsrc = c->S; h.time = c->time;
    h.payload_bytes = buf.size();
    h.checksum = fnv1a(buf.data(), buf.size(), 1469598103934665603ULL);
    std::string tmp = std::string(path) + ".tmp";
    FILE* f = fopen(tmp.c_str(), "wb");
    if (!f) return fail(c, SPARC_EIO, std::string("cannot open ") + tmp);
    bool ok = fwrite(&h, sizeof(h), 1, f) == 1 && fwrite(buf.data(), 1, buf.size(), f) == buf.size();
    ok = (fclose(f) == 0) && ok;
    if (!ok || rename(tmp.c_str(), path) != 0) return fail(c, SPARC_EIO, "checkpoint write failed");
    return SPARC_OK;
}

int sparc_gpu_restore(sparc_ctx* c, const char* path) {
    if (!c || !path) return SPARC_EINVAL;
    if (c->mhd) return fail(c, SPARC_EINVAL, "checkpoints hold the quiet-Sun state layout (not the MHD forms)");
    if (!c->have_bg) return fail(c, SPARC_ESTATE, "set_background first");
    FILE* f = fopen(path, "rb");
    if (!f) return fail(c, SPARC_EIO, std::string("cannot open ") + path);
    CkHeader h;
    if (fread(&h, sizeof(h), 1, f) != 1 || memcmp(h.magic, "SPARCGPU", 8) != 0) {
        fclose(f);
        return fail(c, SPARC_EIO, "not a checkpoint file");
    }
    size_t na = (size_t)c->S * c->nf * c->fs * csz(c), np = (size_t)c->S * 2 * c->ps * csz(c);
    if (h.abi != SPARC_GPU_ABI_VERSION || h.nx != c->P.nx || h.ny != c->P.ny || h.nz != c->nz ||
        h.npmlbot != c->P.npmlbot || h.npmltop != c->P.npmltop || h.option != c->P.option ||
        h.precision != c->P.precision || h.nsrc != c->S || h.payload_bytes != na + np || h.time < 0) {
        fclose(f);
        return fail(c, SPARC_EIO, "checkpoint does not match this context");
    }
    std::vector<unsigned char> buf(na + np);
    size_t got = fread(buf.data(), 1, buf.size(), f);
    fclose(f);
    if (got != buf.size()) return fail(c, SPARC_EIO, "checkpoint truncated");
    if (fnv1a(buf.data(), buf.size(), 1469598103934665603ULL) != h.checksum)
        return fail(c, SPARC_EIO, "checkpoint checksum mismatch");
    CK(cudaMemcpyAsync(c->a, buf.data(), na, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->pml, buf.data() + na, np, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemsetAsync(c->scr, 0, na, c->stream));
    CK(cudaMemsetAsync(c->scrpml, 0, np, c->stream));
    c->t0.assign(c->S, 0);
    CK(cudaMemsetAsync(c->d_t0, 0, (size_t)c->S * sizeof(int), c->stream));
    CK(cudaStreamSynchronize(c->stream));
    c->time = h.time;
    launch_set_time(c->d_time, c->time, c->stream);
    return SPARC_OK;
}

}  // extern "C"
