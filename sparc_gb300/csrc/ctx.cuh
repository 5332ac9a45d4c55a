// Private: the context behind the C ABI, shared by the translation units that
// implement it (capi.cu, mhd.cu), and the error / allocation helpers they use.
#pragma once
#include <string>
#include <vector>
#include "internal.cuh"
#include "../../include/sparc_gpu.h"

static inline double R4(double x) { return (double)(float)x; }

struct MhdState;    // magnetic (option 10) background and stage scratch, mhd.cu

struct sparc_ctx {
    sparc_params P;
    int H, M, nz, S, nzpml;
    long long fs, ps, NP, N;
    int f32;
    int nf;                 // fields per state slot: 6, or 8 in the MHD velocity form (option 8)
    cudaStream_t stream = nullptr;
    cudaEvent_t ev_done = nullptr;     // last cross-context hand-off on this stream
    std::string err;
    long long launches = 0;
    long long dev_bytes = 0;
    std::vector<void*> allocs;

    // host set-up (FP64)
    bool have_bg = false;
    double pi, rsun, normx, normy, dimc, dimrho, diml, deltat, stretchx, stretchy, delta_width;
    double betas[5];
    int e_rad, o_rad, steps, freq_filtering, maxtime, forcing_length, cadforcing_step, num_steps;
    std::vector<double> zt_host;     // ZT_COUNT * nz
    std::vector<double> zq, cq, rhoq; // z, c, rho of the quiet column (non-dimensional; option 10 set-up)
    std::vector<double> pt_host;     // PT_COUNT * M
    Compact<double> cc64;
    int time = 0;

    // device state (element type T; CT = T2)
    void* a = nullptr; void* scr = nullptr; void* pml = nullptr; void* scrpml = nullptr;
    void* ybuf = nullptr; void* pbuf = nullptr; void* rbuf = nullptr;
    void* zt = nullptr; void* pt = nullptr;       // T tables
    float* ftab = nullptr;                        // fused FP32 step: z table [FZ_COUNT][fused_nzp(nz)]
    int use_fused = 0;
    int fused_pencils = 4;                        // modes per CTA of the fused step (autotuned)
    int fused_test_nocopy = 0;                    // test switch: the fused step's table copy is not issued
    int stage_block = 128;                        // threads per CTA of the per-stage kernels (autotuned)
    int stage_q = 1, stage_chunk = 0;             // FP64 stage: lanes per pencil and levels per lane
    void* zc = nullptr;                           // their chunk products of the multipliers (4 rows of nz)
    double* zt64 = nullptr; double* pt64 = nullptr;
    double* tw_x = nullptr; double* tw_y = nullptr;
    void* tmp = nullptr;          // FFT intermediate, nz*M complex T
    void* phys = nullptr;         // one physical field, N reals T
    double* phys64 = nullptr;     // N doubles
    double2* spec64 = nullptr;    // nz*M complex double (primitives)
    double2* spec64b = nullptr;
    double2* tmp64 = nullptr;
    int* d_flag = nullptr;
    void* src_plane = nullptr;    // [S][M] float2: the fused step's interpolated source plane
    int rhs_out = 1;              // the last step of each step call leaves its right-hand side in scr

    // sources
    int src_mode = 0;
    int src_L = 0;
    void* planes = nullptr;       // [S][L][M] CT
    double* series = nullptr;     // [S][nseries]
    int nseries = 0;
    std::vector<int> src_set;

    // surface records
    int rec_on = 0, rec_max = 0;
    void* rec = nullptr;          // [S][rec_max][M] CT, record r = output at slot time r*steps
    // per-slot clocks (continuous batching)
    int* d_t0 = nullptr;          // [S] device copy
    int* d_time = nullptr;        // device copy of `time`, read by the step kernels
    // captured step sequences, replayed as CUDA graphs: one per step count,
    // valid while no kernel argument changed (epoch)
    struct GraphEntry { int n; long long epoch; cudaGraphExec_t exec; long long nlaunch; };
    std::vector<GraphEntry> graphs;
    long long epoch = 0;
    int use_graphs = 1;
    std::vector<int> t0;          // slot time = time - t0[slot]
    int active_n = 0;             // slots 0..active_n-1 are stepped

    // device-resident checkpoints (a + PML + time of every slot)
    void* dck = nullptr; int dck_n = 0;
    std::vector<int> dck_time;
    // kernels
    void* store = nullptr; int store_n = 0;     // [nsnap][7][S][N] T (field-major within a snapshot)
    // per store slot: recorded on the adjoint stream after its reads of the
    // slot; a later snapshot into the slot waits for it
    std::vector<cudaEvent_t> slot_ev;
    std::vector<char> slot_pending;
    double* kacc = nullptr;                     // [S][3][N]
    void* ktemp = nullptr;                      // [7][G][N] T, G = kernel_group(S)
    void* gtmp = nullptr;                       // [G] spectral fields: transform scratch of a source group
    // option 10: the state is physical ([src][field] slots of fs complex
    // elements each hold one dense (nz, ny, nx) real field)
    MhdState* mhd = nullptr;
    // model update (grad.py): three N-point FP64 fields, the filterx
    // multiplier (M) and reduction scratch, allocated on first use
    double* upd = nullptr;
};


static inline int fail(sparc_ctx* c, int code, const std::string& msg) {
    if (c) c->err = msg;
    return code;
}

#define CK(call)                                                                   \
    do {                                                                           \
        cudaError_t e_ = (call);                                                   \
        if (e_ != cudaSuccess)                                                     \
            return fail(c, SPARC_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

#define CKL()                                                                      \
    do {                                                                           \
        cudaError_t e_ = cudaGetLastError();                                       \
        if (e_ != cudaSuccess)                                                     \
            return fail(c, SPARC_ECUDA, std::string("kernel launch: ") + cudaGetErrorString(e_)); \
    } while (0)

static inline int dalloc(sparc_ctx* c, void** p, size_t bytes) {
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        *p = nullptr;
        cudaGetLastError();
        return fail(c, SPARC_ENOMEM, "cudaMalloc of " + std::to_string(bytes) + " bytes failed: " + cudaGetErrorString(e));
    }
    c->allocs.push_back(*p);
    c->dev_bytes += (long long)bytes;
    cudaMemsetAsync(*p, 0, bytes, c->stream);
    return SPARC_OK;
}

static inline int upload(sparc_ctx* c, void* dst, const void* src, size_t bytes) {
    CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, c->stream));
    return SPARC_OK;
}

static inline size_t esz(const sparc_ctx* c) { return c->f32 ? sizeof(float) : sizeof(double); }
static inline size_t csz(const sparc_ctx* c) { return 2 * esz(c); }
template <typename T> typename CplxOf<T>::type* CP(void* p) { return (typename CplxOf<T>::type*)p; }

// option 10 (mhd.cu)
int mhd_create(sparc_ctx* c);
void mhd_destroy(sparc_ctx* c);
int mhd_set_stream_priority(sparc_ctx* c, int cuda_priority);   // the second stream's priority
int mhd_set_background(sparc_ctx* c, const double* rho, const double* cs, const double* p, const double* bx,
                       const double* by, const double* bz);
int mhd2d_set_background(sparc_ctx* c, const double* p, const double* rho, const double* cs, const double* psi);
int mhd_steps(sparc_ctx* c, int nsteps);
// sensitivity kernels of option 18 (mhd.cu)
int mhd2d_derive(sparc_ctx* c, int s0, int G, bool adjoint, void* out, long long ofs);
int mhd2d_kernel_b_reset(sparc_ctx* c);
int mhd2d_kernel_b_accumulate(sparc_ctx* c, const void* fst, long long sfs, const void* adj, long long afs, int s0,
                              int G);
int mhd2d_kernels_b(sparc_ctx* c, int src, int sum_slots, double* kbx, double* kbz, double* kpsi);
const double* mhd_kernel_c2(const sparc_ctx* c);    // per-point c^2 and rho0 of a 2-D MHD context, or null
const double* mhd_kernel_rho0(const sparc_ctx* c);
void* mhd_pml(sparc_ctx* c);      // [S][6][nzpml*NP] T pmlvars of option 10
void* mhd_spml(sparc_ctx* c);     // scrpml
