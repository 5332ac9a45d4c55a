/*
 * sparc_gpu.h -- C ABI of the GB300 (sm_103a) SPARC time-stepping library.
 *
 * The reference (jishnub/sparc) has no plugin or FFI layer: its hot path is the
 * `call step()` seam inside the Fortran TIMESTEPPING loop (driver.f90:424),
 * operating on module globals (initialize.f90:24-153), and the outside world
 * reaches it only through `mpiexec -np 1 ./sparc <src> <ls>` plus files
 * (full.py:49,67; linesearch.py:47-52; data_forward.py:49-52).  Each entry
 * point below names the reference routine (file:line) whose job it takes over.
 *
 * Conventions
 *   - Every entry point returns an int status (SPARC_OK = 0, negative on error)
 *     and never exits or traps.  sparc_gpu_errstr() describes a status and
 *     sparc_gpu_last_error() the last failure of a context in words.
 *   - Host arrays are FP64 and caller-owned; the library copies in and out and
 *     keeps no host pointer beyond a call.  Device memory belongs to the
 *     context.
 *   - 3-D fields are laid out as the reference's Fortran arrays a(nx,ny,nz):
 *     x fastest, then y, then z  (C order [nz][ny][nx]).
 *   - One context per host thread; calls on one context must be serialised by
 *     the caller.  Contexts are independent (one CUDA stream each).
 */
#ifndef SPARC_GPU_H
#define SPARC_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

#define SPARC_GPU_ABI_VERSION 1

/* status codes */
#define SPARC_OK 0
#define SPARC_EINVAL (-1)     /* bad parameter or argument */
#define SPARC_ENOMEM (-2)     /* device or host allocation failed */
#define SPARC_ECUDA (-3)      /* a CUDA call failed */
#define SPARC_ETIMEDOUT (-4)  /* a bounded device wait gave up */
#define SPARC_ENAN (-5)       /* non-finite values detected in the state */
#define SPARC_ESTATE (-6)     /* call out of order (e.g. no background yet) */
#define SPARC_EIO (-7)        /* file read/write failed or corrupt */

/* precision of the bulk field arithmetic */
#define SPARC_FP64 0          /* plain: everything FP64 */
#define SPARC_FP32 1          /* FP32 fields; FP64 set-up, profiles and kernel accumulation */

/* source modes for sparc_gpu_set_source */
#define SPARC_SRC_NONE 0
#define SPARC_SRC_SERIES 1    /* forcing(t) = plane[0] * series[time]        (physics2d.f90:1066) */
#define SPARC_SRC_LAGRANGE 2  /* forcing(t) = 7-point Lagrange interpolation of planes sampled
                                 every cadforcing seconds (LAGRANGE_INTERP, physics.f90:678-737) */

/* field indices of the displacement form (initialize.f90:515-527) */
#define SPARC_XI_X 0
#define SPARC_XI_Y 1
#define SPARC_XI_Z 2
#define SPARC_V_X 3
#define SPARC_V_Y 4
#define SPARC_V_Z 5

/* Mirror of params.i (params.i:25-150) plus the Instruction-file flags
 * (initialize.f90:1006-1051).  Lengths in cm, times in s, frequencies in Hz. */
typedef struct sparc_params {
    int nx, ny, nz;            /* params.i:25  (nx, ny powers of two; ny = 1 for options 17, 18) */
    int npmlbot, npmltop;      /* params.i:108 */
    int option;                /* step.f90:74-110: 2 = MP_QUIET_PML_3D, 4 = MP_QUIET_PML_3D_DISPL,
                                  8 = MP_MHD_PML_3D, 10 = MP_MHD_PML_3D_DISPL,
                                  17 = MP_QUIET_PML_2D_DISPL, 18 = MP_MHD_PML_2D_DISPL */
    int compute_forward;       /* Instruction 'spectral' */
    int compute_adjoint;       /* Instruction 'adjoint' */
    int damp_waves;            /* params.i:38 */
    int src_k;                 /* 1-based source plane; 0 = e_rad (forward) / o_rad (adjoint) */
    int precision;             /* SPARC_FP64 or SPARC_FP32 */
    int nsrc;                  /* number of sources on the source axis (batch) */
    double xlength, ylength, timestep;   /* params.i:26 */
    double excitdep, obsheight;          /* params.i:150, :130 */
    double cadforcing, outputcad;        /* params.i:47, :136 */
    double nupeak, nuwidth;              /* params.i:64 */
    double solartime;                    /* params.i:129 (hours) */
} sparc_params;

typedef struct sparc_ctx sparc_ctx;

/* ---- life cycle ---------------------------------------------------------- */

/* Replaces Initialize_all (initialize.f90:165-583): validates p, picks the
 * device's current GPU, allocates all device state.  *out is NULL on error. */
int sparc_gpu_create(const sparc_params* p, sparc_ctx** out);

/* Releases device memory and the stream.  Accepts NULL. */
void sparc_gpu_destroy(sparc_ctx* ctx);

const char* sparc_gpu_errstr(int status);
const char* sparc_gpu_last_error(const sparc_ctx* ctx);
int sparc_gpu_abi_version(void);

/* ---- set-up -------------------------------------------------------------- */

/* Replaces solar_data (initialize.f90:728-774), the stretch set-up
 * (initialize.f90:464-472), mp_Initialize_RHS / _2d (physics.f90:34-404,
 * physics2d.f90:23-410), INIT_DAMPING (damping.f90:10-120) and
 * INITIALIZE_STEP (step.f90:24-41).  Inputs are the six columns of the
 * background file, one value per z-level, bottom first, in cgs units:
 * z = r/R_sun, c, rho, p, g, Gamma_1.  All set-up arithmetic is FP64.
 * Resets the state to zero and the time index to 0. */
int sparc_gpu_set_background(sparc_ctx* ctx, const double* z, const double* c,
                             const double* rho, const double* p0, const double* g,
                             const double* gamma1);

/* Source of source-axis slot src_idx.  planes: L horizontal planes (ny,nx),
 * series: nseries values indexed by the time-step index (SPARC_SRC_SERIES).
 * For SPARC_SRC_LAGRANGE the planes are vr(:,:,1..L) of LAGRANGE_INTERP
 * sampled every cadforcing seconds and series is ignored.  Replaces the
 * source set-up of DETERMINE_STATUS (driver.f90:591-695). */
int sparc_gpu_set_source(sparc_ctx* ctx, int src_idx, int mode, const double* planes, int L,
                         const double* series, int nseries);

/* ---- time stepping --------------------------------------------------------- */

/* nsteps iterations of the TIMESTEPPING body (driver.f90:412-424): forcing
 * interpolation, STEP (step.f90:43-128: five LDDRK stages of the selected RHS,
 * PML auxiliaries, FILTER_VARS_3D / _2D), then time = time + 1.  When surface
 * recording is on, vz at o_rad is recorded whenever mod(time, steps) == 0
 * (driver.f90:455-476). */
int sparc_gpu_step(sparc_ctx* ctx, int nsteps);

/* Options 10 (MP_MHD_PML_3D_DISPL, displacement.f90:663-849) and 8
 * (MP_MHD_PML_3D, pml.f90:80-208): the 3-D cgs background that READ_IN_FIELD reads (all_modules.f90:486-513) -- density,
 * sound speed, pressure and B_x, B_y, B_z, each nx*ny*nz values in the
 * Fortran order a(nx,ny,nz) -- after sparc_gpu_set_background has set the
 * quiet column (z grid, gravity, Gamma_1, and the column the source planes
 * are searched on).  Replaces the magnetic parts of mp_Initialize_RHS
 * (physics.f90:62-161, 204-208, 255-303, 356-363).  For both options the
 * state is physical (get_field / get_state return it without transforms) and
 * the PML arrays of set_state / get_state hold six auxiliaries (psi_vz,
 * psi_p, psi_dzbx, psi_dzby, psi_induction_bx, psi_induction_by) of nzpml
 * planes: option 10 accounts for the bottom layer only, option 8 for both.
 * Option 8 holds eight fields per state (rho, v_x, v_y, v_z, p, b_x, b_y,
 * b_z; initialize.f90:498-510,545-551). */
int sparc_gpu_set_mhd_background(sparc_ctx* ctx, const double* rho, const double* c, const double* p,
                                 const double* bx, const double* by, const double* bz);

/* Option 18 (MP_MHD_PML_2D_DISPL, physics2d.f90:724-943; ny = 1): the 2-D
 * cgs background -- density, sound speed, pressure and the vector potential
 * psi (model_vectorpsi), each nx*nz values a(nx,nz) -- after
 * sparc_gpu_set_background.  B_x = -d psi/dz and B_z = d psi/dx * stretchx
 * (DBYD1 with ibc 0) as the magnetic part of mp_Initialize_RHS_2d forms them
 * (physics2d.f90:106-195), then the gradients, the PML at both ends with the
 * magnetic wave speed and the source planes e_rad / o_rad (:223-341).  The
 * state is physical and the PML arrays of set_state / get_state hold six
 * auxiliaries of nzpml planes (psi_vz, psi_p, psi_dzbx, unused, psi_induction_bx,
 * unused). */
int sparc_gpu_set_mhd2d_background(sparc_ctx* ctx, const double* rho, const double* c, const double* p,
                                   const double* psi);

/* Pick the fastest of the launch variants that give identical results (the
 * fused FP32 step's modes per CTA, 4 or 2; the per-stage kernels' threads per
 * CTA, 128 or 64) by timing real steps: the call advances the solution by
 * 4*steps ordinary time steps.  Steps are replayed from captured CUDA graphs
 * (one per step count, captured on first use and after any change of launch
 * arguments); SPARC_NO_GRAPHS in the environment at create time launches
 * them directly.  choice / ms_per_step may be NULL.  No reference
 * counterpart (tuning of this implementation). */
int sparc_gpu_autotune(sparc_ctx* ctx, int steps, int* choice, float* ms_per_step);

/* One RK stage rk = 1..5 of the current step (one pass of the do step_rk
 * loop body, step.f90:49-112) without the update, the filters or a time
 * advance: a fine-grained seam for timing the stage kernel on its own. */
int sparc_gpu_stage(sparc_ctx* ctx, int rk);

int sparc_gpu_get_time(const sparc_ctx* ctx, int* time);
int sparc_gpu_set_time(sparc_ctx* ctx, int time);

/* ---- state in and out ------------------------------------------------------ */

/* Field `field` (SPARC_XI_X..SPARC_V_Z) of slot src_idx into host (nz,ny,nx),
 * or only plane k (1-based) into host (ny,nx) when k > 0.  With nf fields
 * per state (6; 8 in option 8), field nf..2nf-1 return the last RK-stage
 * right-hand side scr(:,:,:,1..nf); in the displacement forms components
 * 4..6 of it are the 'acc' fields of WRITE_OUT_PARTIAL_STATE
 * (all_modules.f90:771-778). */
int sparc_gpu_get_field(sparc_ctx* ctx, int src_idx, int field, int k, double* host);

/* Whole state of one slot: a (nf,nz,ny,nx) -- nf = 6, or 8 in option 8 --
 * and the PML auxiliaries pmlvars (2,nzpml,ny,nx), or (6,nzpml,ny,nx) in the
 * MHD forms; pml may be NULL.  Replaces READ_IN_INITIAL_CONDITION /
 * WRITE_OUT_FULL_STATE (all_modules.f90:533-694) in memory. */
int sparc_gpu_set_state(sparc_ctx* ctx, int src_idx, const double* a, const double* pml);
int sparc_gpu_get_state(sparc_ctx* ctx, int src_idx, double* a, double* pml);

/* Surface seismogram recording (the vz_cc.bin stream, driver.f90:455-476):
 * enable with room for max_records outputs per slot; record r of a slot is vz
 * at o_rad after the step at slot time r*steps.  Fetch them as (nrec,ny,nx)
 * FP64 records, the layout of write_binary_seq_2D (all_modules.f90:947-1006);
 * nrec counts the outputs the slot has reached so far. */
int sparc_gpu_record_surface(sparc_ctx* ctx, int enable, int max_records);
int sparc_gpu_get_records(sparc_ctx* ctx, int src_idx, double* host, int* nrec);

/* ---- continuous batching ---------------------------------------------------- */

/* Every slot runs its own clock, slot time = context time - (context time at
 * its last reset).  The source series index, LAGRANGE_INTERP, the horizontal
 * filter cadence and the output cadence follow the slot time, so a request
 * admitted into a free slot of a running batch starts at time 0 while sharing
 * the batch's launches.  slot_reset clears the slot's state, PML, scr and
 * records and restarts its clock at 0; its source stays as set. */
int sparc_gpu_slot_reset(sparc_ctx* ctx, int src_idx);
int sparc_gpu_slot_time(const sparc_ctx* ctx, int src_idx, int* slot_time);

/* Only slots 0..nactive-1 are stepped (default: all). */
int sparc_gpu_set_active(sparc_ctx* ctx, int nactive);

/* Whether the last step of each sparc_gpu_step call leaves that step's
 * right-hand side in scr (default 1).  scr is what get_field returns for
 * fields nf..2nf-1, and the forward kernel snapshot reads it (f_acc,
 * kernels.f90:197-263), so sparc_gpu_snapshot fails with SPARC_ESTATE while it
 * is 0.  An adjoint context of the kernel workflow reads no scr; turning the
 * output off there saves the fused FP32 step one full-state write per call.
 * The state itself does not depend on it.  No counterpart in the reference,
 * which keeps scr in memory at all times (step.f90:24-128). */
int sparc_gpu_set_rhs_output(sparc_ctx* ctx, int on);

/* Scheduling priority of the context's stream(s): level 0 is the default
 * (least urgent), each level above it one step more urgent, clamped to the
 * device's range.  The context waits for its queued work and moves to new
 * streams, so call it between steps.  When contexts share a GPU, the
 * scheduler starts the CTAs of more urgent streams first: a serving loop
 * gives its cheap requests' contexts the higher levels.  No counterpart in
 * the reference (one MPI process per source). */
int sparc_gpu_set_stream_priority(sparc_ctx* ctx, int level);

/* Non-blocking: *busy = 1 while work queued on the context's stream has not
 * finished, 0 once it has (cudaStreamQuery). */
int sparc_gpu_query(sparc_ctx* ctx, int* busy);

/* Checkpoint / restore of every slot (state, PML, time) to one file with a
 * checksum; restore rejects a corrupt or mismatching file with SPARC_EIO.
 * A restore restarts every slot clock at the restored time index. */
int sparc_gpu_checkpoint(sparc_ctx* ctx, const char* path);
int sparc_gpu_restore(sparc_ctx* ctx, const char* path);

/* Device-resident copies of the whole state (a, PML auxiliaries, time index)
 * of every slot, in `capacity` slots allocated by the first save; used to
 * recompute forward segments in reverse order for the kernel integral,
 * whose forward and adjoint snapshots pair in reversed time
 * (kernels.f90:203,241).  Loading clears scr. */
int sparc_gpu_save_device(sparc_ctx* ctx, int idx, int capacity);
int sparc_gpu_load_device(sparc_ctx* ctx, int idx);

/* ---- sensitivity kernels (kernels.f90:197-311, 523-539) ------------------- */

/* The forward-snapshot store: saves the spectral quantities that the kernel
 * integral needs from the current state of forward context `fwd` into slot
 * `snap` (0-based) of the store.  Allocates the store on first use for
 * nsnap snapshots. */
int sparc_gpu_snapshot(sparc_ctx* fwd, int snap, int nsnap);

/* One accumulation of kernels.f90:276-311 for every slot: forward snapshot
 * `snap` of `fwd` against the current state of adjoint context `adj`.
 * Accumulators are FP64 and live in `adj`.  The two contexts' streams are
 * ordered by events: the accumulation waits for the snapshot, and later work
 * on `fwd` waits for the accumulation (so the store slot may be reused). */
int sparc_gpu_kernel_accumulate(sparc_ctx* fwd, int snap, sparc_ctx* adj);

/* Resets the accumulators of `adj`. */
int sparc_gpu_kernel_reset(sparc_ctx* adj);

/* Final scaling (kernels.f90:523-539) into host arrays (nz,ny,nx): K_c, K_rho,
 * hessian of slot src_idx (sum_slots != 0: summed over the source axis,
 * the grad.py:158-165 sum). */
int sparc_gpu_kernels(sparc_ctx* adj, int src_idx, int sum_slots, double* kc, double* krho,
                      double* hessian);

/* The same final scaling into a caller-owned DEVICE buffer of 3*nx*ny*nz
 * doubles: K_c, K_rho, hessian, each (nz,ny,nx).  The work is enqueued on
 * the context's stream (sparc_gpu_stream) and the call returns without
 * waiting: a caller that reads `dev_out` from another stream orders it after
 * that stream first.  This is the form a multi-GPU driver sums across ranks
 * with one FP64 all-reduce in device memory (grad.py:158-165 sums the
 * per-source kernel files on the host). */
int sparc_gpu_kernels_device(sparc_ctx* adj, int src_idx, int sum_slots, double* dev_out);

/* Option 18 (2-D MHD): the B-field kernels of the MAGNETIC_KERNELS block
 * (kernels.f90:337-453) accumulated beside K_c, K_rho and the hessian, with
 * B0 and curl B0 formed as kernel mode forms them from the vector potential
 * (kernels.f90:99-133), scaled as kernels.f90:498-514 into host arrays
 * (nz,1,nx): kernel_bx, kernel_bz and kernel_vectorpsi (the y component of
 * the curl of (kernel_bx, 0, kernel_bz)).  Any of the three may be NULL. */
int sparc_gpu_kernels_b(sparc_ctx* adj, int src_idx, int sum_slots, double* kbx, double* kbz, double* kpsi);

/* ---- adjoint source of a 2-D run (ADJOINT_SOURCE_FILT) -------------------- */

typedef struct {
    double x00;            /* master pixel x (Mm) of this source (data/master.pixels) */
    double t1_min;         /* first output time in minutes: the timeline reversed and negated,
                              divided by 60 (driver.f90:1310-1315) */
    double dt_min;         /* output cadence in minutes */
    int have_ridge[3];     /* params.0 (f ridge), params.1 (p1 ridge), params.2 (band-passed set) exist */
    double ridge[3][3];    /* per set: mindist (Mm), maxdist (Mm), window (min) */
    int have_band[2];      /* filter.params.0 / .1 exist */
    double band[2][2];     /* left, right corner (mHz) */
    int linesearch;        /* 1: windows of sets 0, 1 are read from `windows` (windows.0/.1) */
} sparc_adjsrc_params;

/* ADJOINT_SOURCE_FILT (driver.f90:1262-1686) of a 2-D context (ny = 1): the
 * ridge filters (FMODE_FILTER, PMODE_FILTER, FREQ_FILTER), a window and a
 * COMPUTE_TT travel time per pixel in each set's distance range, and the
 * time-reversed adjoint source, computed on the GPU from the surface records
 * of slot src_idx (the synthetic vz_cc, first nt records) and the observed
 * data (nt, nx) from the host.  windows: int[2][nx][2], (lef, rig) per pixel
 * of sets 0 and 1, 1-based, 0 for no measurement (written, or read when
 * linesearch).  adj: (nt, nx), the source.fits of the adjoint run; misfit =
 * 0.5 sum tau^2 and nmeas as the kernel/misfit file (driver.f90:1668-1674). */
int sparc_gpu_adjoint_source(sparc_ctx* ctx, int src_idx, const double* data, int nt,
                             const sparc_adjsrc_params* ap, int* windows, double* adj, double* misfit,
                             int* nmeas);

/* The same from a synthetic (nt, nx) in host memory (a vz_cc.fits read from
 * disk, as the reference reads it) instead of the context's records. */
int sparc_gpu_adjoint_source_host(sparc_ctx* ctx, const double* synth, const double* data, int nt,
                                  const sparc_adjsrc_params* ap, int* windows, double* adj, double* misfit,
                                  int* nmeas);

/* MISFIT_ALL (driver.f90:1702-2076) of a 2-D run, the line search's misfit:
 * for the bands 2-3.5, 3.5-4.5 and 4.5-6 mHz, the three sets of
 * sparc_gpu_adjoint_source (ap's ridges; its bands are not used) with
 * MISFIT_ALL's ridge speeds and arrival polynomial.  synth: the synthetic
 * (nt, nx) on the host, or NULL for the records of slot src_idx.  windows:
 * int[3][2][nx][2], the band's sets 0 and 1 (windows.all.N), written or read
 * (ap->linesearch); misfit: double[3][3] = 0.5 sum tau^2 and nmeas:
 * int[3][3] per band and set (kernel/misfit_all_XX_YY). */
int sparc_gpu_misfit_all(sparc_ctx* ctx, int src_idx, const double* synth, const double* data, int nt,
                         const sparc_adjsrc_params* ap, int* windows, double* misfit, int* nmeas);

/* ---- model update of an inversion iteration (grad.py) --------------------- */

/* Replaces grad.py:152-186 (the kernel sums are the caller's, as grad.py
 * reads them from the kernel_*.fits files).  Host arrays (nz,ny,nx) of the context's
 * grid, FP64: kc_sum = sum of kernel_c, kpsi_sum = sum of kernel_vectorpsi,
 * hess_sum = sum of |hessian| over the sources; rho_z[nz] the density
 * column of the background (the third column of the polytrope file).
 * hess = max(hess_sum rho_z / max, 5e-3); grad_c = filterz 'smooth' of
 * filterx(kc_sum / hess); grad_psi = gaussian_filter1d along z (sigma 2,
 * reflect) of antisymmetrize(filterx(kpsi_sum / hess)).  Either output may
 * be NULL (its kernel sum may then be NULL).  Needs set_background. */
int sparc_gpu_gradient(sparc_ctx* ctx, const double* kc_sum, const double* kpsi_sum, const double* hess_sum,
                       const double* rho_z, double* grad_c, double* grad_psi);

/* Replaces grad.py:188-301 (steepest descent and conjugate gradient; the
 * LBFGS branch there is switched off and names an undefined variable).
 * last_grad_psi NULL: steepest descent, update = gradient, *con = 0.  Else
 * conjugate gradient: con = max(0, sum g (g - g_last) / sum g_last^2) of the
 * vectorpsi gradients, update = gradient + con * last update (last_update_psi
 * and, when update_c is asked for, last_update_c required).  With nmodels >
 * 0 writes test_psi[nmodels][nz*ny*nx], model i+1 = model_psi + eps (i+1)
 * rms(model_psi) update_psi / max|update_psi| (grad.py uses eps 1e-7 and 5
 * models).  update_c, update_psi and con may be NULL. */
int sparc_gpu_update_models(sparc_ctx* ctx, const double* grad_c, const double* grad_psi,
                            const double* last_grad_psi, const double* last_update_c,
                            const double* last_update_psi, const double* model_psi, double eps, int nmodels,
                            double* update_c, double* update_psi, double* test_psi, double* con);

/* ---- primitives (the reference's derivative routines) ---------------------- */

/* ddx / ddy (derivatives.f90:28-170) and ddz (derivatives.f90:10-24 with
 * DBYD2 dbyd2.f90:8-237 + MTRIDAG mtridag.f90:94-111) of one host field
 * (nz,ny,nx) using the context's grid; bc as in DBYD2 (0..3).  For bc 2 / 3
 * dvar must carry the caller-set boundary plane (k = 1 / k = nz) on input. */
int sparc_gpu_ddx(sparc_ctx* ctx, const double* var, double* dvar);
int sparc_gpu_ddy(sparc_ctx* ctx, const double* var, double* dvar);
int sparc_gpu_ddz(sparc_ctx* ctx, const double* var, double* dvar, int bc);

/* damp_velocity (damping.f90:125-161) of one field: rhs -= damping(v). */
int sparc_gpu_damp(sparc_ctx* ctx, const double* v, double* rhs);

/* ---- measurement hooks ------------------------------------------------------ */

/* The context's CUDA stream (a cudaStream_t), for event timing by the caller. */
void* sparc_gpu_stream(sparc_ctx* ctx);

/* Number of kernels this context has launched so far. */
long long sparc_gpu_launch_count(const sparc_ctx* ctx);

/* Device bytes held by the context. */
long long sparc_gpu_device_bytes(const sparc_ctx* ctx);

/* Set-up diagnostics: info[0..14] = e_rad, o_rad, delta_width, deltat,
 * steps, freq_filtering, maxtime, forcing_length, cadforcing_step, num_steps,
 * betas(1..5); ztab / ptab receive the FP64 z-profile and pencil tables
 * (either may be NULL): ztab holds SPARC_ZTAB_ROWS rows of nz values, ptab
 * SPARC_PTAB_ROWS rows of ny*(nx/2+1) values. */
#define SPARC_ZTAB_ROWS 25
#define SPARC_PTAB_ROWS 4
int sparc_gpu_info(sparc_ctx* ctx, double* info, double* ztab, double* ptab);

/* Blocks until the context's stream is idle; SPARC_ENAN if check_finite and
 * the state of any slot holds a non-finite value. */
int sparc_gpu_sync(sparc_ctx* ctx, int check_finite);

/* ---- no-allocation entry point ---------------------------------------------- */

/* Spectral -> physical transform of nplanes horizontal planes that allocates
 * nothing.  This entry point has no counterpart in the reference.
 *
 * It is for callers that cannot call cudaMalloc while they run: an
 * application whose pool already owns the rest of HBM (any further
 * cudaMalloc fails), or an output thread that must not make cudaMalloc /
 * cudaFree synchronise the device under solves running on other streams.
 * The caller passes its own device buffers:
 *   spec  nplanes x ny x (nx/2+1) complex values of the context's precision
 *         (double2 for SPARC_FP64, float2 for SPARC_FP32), the normalised
 *         r2c half-spectrum in which the library keeps its state
 *         (= rfft2(plane) / (nx*ny));
 *   phys  nplanes x ny x nx reals of the context's precision (output).
 * The work is queued on `stream` (a cudaStream_t; NULL = the context's
 * stream) and the call returns without waiting for it.
 *
 * Scratch: one fixed 32 MiB device array inside the library (held by every
 * GPU that loads it until the process exits).  A call needing more than
 * that -- nplanes * ny * (nx/2+1) complex values when ny > 1 -- is rejected
 * with SPARC_EINVAL and a message giving the largest allowed nplanes; split
 * such work over several calls.  The first call on a device looks up the
 * array's device address with that device current, so make the first call
 * on each device before any stream capture.  All calls share the array:
 * calls that overlap on the GPU (different streams or threads) race and
 * must be serialised by the caller. */
int sparc_gpu_spec_to_phys_noalloc(sparc_ctx* ctx, const void* spec, void* phys, int nplanes,
                                   void* stream);

#ifdef __cplusplus
}
#endif
#endif /* SPARC_GPU_H */
