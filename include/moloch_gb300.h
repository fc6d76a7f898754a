/*
 * moloch_gb300.h -- C ABI of the GB300-native MOLOCH dynamical-core step.
 *
 * This is the drop-in boundary for the reference's Fortran module
 * `mod_moloch` (nompi/mod_moloch.F90), whose public interface is
 *     public :: allocate_moloch , init_moloch , moloch        (:93)
 * A replacement `mod_moloch` written with ISO_C_BINDING keeps those three
 * names and forwards to the functions below.
 * All arrays cross the boundary as plain host pointers to the Fortran arrays
 * (column-major, j fastest) together with their lower and upper bounds, so
 * the library can check the layout contract of nompi/mod_atmosphere.F90:104-169
 * and nompi/mod_moloch.F90:183-217.  No PyTorch or CUDA types appear here;
 * the only CUDA object is an optional stream passed as `void*`.
 *
 * Every function returns 0 on success or one of the MOLOCH_ERR_* codes; the
 * text of the last error of the calling thread is in moloch_gpu_last_error().
 * A handle owns one CUDA stream and is not re-entrant (the reference is a
 * single-threaded program).
 */
#ifndef MOLOCH_GB300_H
#define MOLOCH_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes -------------------------------------------------------- */
#define MOLOCH_OK 0
#define MOLOCH_ERR_ARG 1      /* bad argument, size or option */
#define MOLOCH_ERR_BOUNDS 2   /* array bounds differ from the layout contract */
#define MOLOCH_ERR_CUDA 3     /* a CUDA call failed */
#define MOLOCH_ERR_CFL 4      /* ps not finite: "CFL VIOLATION" (mod_moloch.F90:402-411) */
#define MOLOCH_ERR_STATE 5    /* call out of order (e.g. step before init) */
#define MOLOCH_ERR_TIMEOUT 6  /* a bounded device wait gave up */
#define MOLOCH_ERR_NOMEM 7    /* device allocation failed */

/* ---- arithmetic modes ---------------------------------------------------- */
#define MOLOCH_FP64 0        /* plain FP64, multiply-add contraction allowed */
#define MOLOCH_FP64_EXACT 1  /* FP64 in the reference's evaluation order, no FMA */
#define MOLOCH_FP32_MIXED 2  /* FP32 storage and stencils, FP64 tridiagonal solve and column sums */

/* ---- field identifiers for upload / download ------------------------------
 * Bounds (j, i, k) with nj = jx, ni = iy follow the reference allocations:
 *   u            (-1:nj+2, 0:ni+1, 1:kz)      mod_atmosphere.F90:107
 *   v            (0:nj+1, -1:ni+2, 1:kz)      :108
 *   t tetav pai  (0:nj+1, 0:ni+1, 1:kz)      :111-114
 *   w            (1:nj, 1:ni, 1:kz+1)         :113
 *   qx           (0:nj+1, 0:ni+1, 1:kz, 1:5)  :115   (MOLOCH_F_QX, 4-D)
 *   qv..qs       the 3-D slices of qx         (mod_moloch.F90:247-251)
 *   zeta         (-1:nj+2, -1:ni+2, 1:kz)     :116
 *   p tvirt qs(qsat) rho  (1:nj, 1:ni, 1:kz)  :118-124
 *   fmz          (0:nj+1, 0:ni+1, 1:kz)       :125
 *   fmzf         (1:nj, 1:ni, 1:kz+1)         :126
 *   ps           (0:nj+1, 0:ni+1)             :166
 *   ht           (-1:nj+2, -1:ni+2)           :131
 *   msfx         (1:nj, 1:ni)                 :140
 *   msfu         (0:nj+1, 1:ni)               :141
 *   msfv         (1:nj, 0:ni+1)               :142
 *   hx           (0:nj+1, 1:ni)               :143
 *   hy           (1:nj, 0:ni+1)               :144
 *   ulat vlat    (1:nj, 1:ni)                 :145,147
 *   zita         (1:kz+1)   zitah (1:kz)      mod_runparams.F90:73-74
 *   s            (1:nj, 1:ni, 1:kz+1)         mod_moloch.F90:190 (download only)
 * The domain is doubly periodic (one rank): halo values passed in are not
 * used, the device recomputes them as periodic images of the interior.
 * Downloads fill the interior; halo positions receive periodic images. */
enum moloch_field {
  MOLOCH_F_U = 0, MOLOCH_F_V, MOLOCH_F_W, MOLOCH_F_PAI, MOLOCH_F_T, MOLOCH_F_TETAV,
  MOLOCH_F_QV, MOLOCH_F_QC, MOLOCH_F_QI, MOLOCH_F_QR, MOLOCH_F_QS,
  MOLOCH_F_QX,    /* 4-D qx(:,:,:,1:5), lb[3] = 1, ub[3] = 5 */
  MOLOCH_F_P, MOLOCH_F_TVIRT, MOLOCH_F_QSAT, MOLOCH_F_RHO, MOLOCH_F_PS,
  MOLOCH_F_ZETA, MOLOCH_F_FMZ, MOLOCH_F_FMZF, MOLOCH_F_HT,
  MOLOCH_F_MSFX, MOLOCH_F_MSFU, MOLOCH_F_MSFV, MOLOCH_F_HX, MOLOCH_F_HY,
  MOLOCH_F_ULAT, MOLOCH_F_VLAT, MOLOCH_F_ZITA, MOLOCH_F_ZITAH,
  MOLOCH_F_S, MOLOCH_F_DELTAW,
  MOLOCH_F_COUNT
};

/* Grid sizes: namelist &dimensions (namelist.in:1-5). */
typedef struct moloch_grid {
  int jx, iy, kz;
} moloch_grid_t;

/* Run parameters set by param() (nompi/regcm_dynamical_core.F90:99-113) and
 * the compile-time switches of mod_moloch (nompi/mod_moloch.F90:95-106),
 * here runtime options with the reference defaults noted. */
typedef struct moloch_params {
  double dt;        /* 30 s */
  double dx;        /* 3000 m */
  double mo_ztop;   /* 36000 m */
  double mo_h;      /* 12000 m */
  double mo_a0;     /* 0 */
  double mo_anu2;   /* 0.6 */
  int mo_nadv;      /* 3 */
  int mo_nsound;    /* 5 */
  int mode;         /* MOLOCH_FP64 | MOLOCH_FP64_EXACT | MOLOCH_FP32_MIXED */
  int mo_divfilter; /* .false. (mod_runparams.F90:55) */
  int do_filterpai; /* .false. (mod_moloch.F90:101) */
  int do_filtertheta; /* .false. (mod_moloch.F90:102) */
  int rotllr;       /* 1: iproj == 'ROTLLR' (mod_dynparam.F90:39) */
} moloch_params_t;

/* Printout of moloch(istep, lprint) (nompi/mod_moloch.F90:395-419) plus
 * the FP64 column sums kept by every mode. */
typedef struct moloch_diag {
  double maxps, minps;  /* Pa, over the interior */
  double maxu, minu, maxv, minv;
  double mass;          /* sum of rho * dz over all points (kg m^-2 summed over columns), FP64 */
  double energy;        /* sum of rho * dz * (cvd*T + g*zeta + (u^2+v^2+w^2)/2), FP64 */
  int status;           /* MOLOCH_OK or MOLOCH_ERR_CFL */
  int nonfinite;        /* number of non-finite ps values */
} moloch_diag_t;

typedef struct moloch_handle moloch_handle_t;

/* allocate_moloch (nompi/mod_moloch.F90:183-217): device arrays for one
 * domain.  `stream` is a cudaStream_t or NULL (the handle then creates one). */
int moloch_gpu_create(const moloch_grid_t* grid, const moloch_params_t* params,
                      void* stream, moloch_handle_t** out);

/* Defaults of moloch_params_t as set by the reference's param(). */
void moloch_gpu_default_params(moloch_params_t* p);

/* Copy one reference array (with its Fortran bounds) to the device.  Part of
 * init_moloch's role (nompi/mod_moloch.F90:219-268, which aliases the module
 * arrays with assignpnt): lb/ub hold the lower/upper bound per dimension. */
int moloch_gpu_upload(moloch_handle_t* h, int field, const double* host_base,
                      const int* lb, const int* ub);

/* init_moloch (nompi/mod_moloch.F90:219-268): derive coru, corv, mx2, rmu,
 * rmv, gzitak, gzitakh, xknu and the static metric terms from the uploaded
 * arrays, set w(:,:,1) = 0.  Call after all uploads. */
int moloch_gpu_init(moloch_handle_t* h);

/* moloch(istep, lprint) (nompi/mod_moloch.F90:272-421): one dt step.
 * With lprint != 0 the max/min of ps, u, v and the column sums are reduced
 * on the device and returned in *diag (may be NULL when lprint == 0); a
 * non-finite ps returns MOLOCH_ERR_CFL, like the reference's fatal() call. */
int moloch_gpu_step(moloch_handle_t* h, int istep, int lprint, moloch_diag_t* diag);

/* Run nsteps steps back to back with no host synchronisation in between
 * (the time loop of nompi/regcm_dynamical_core.F90:49-53 without output).
 * use_graph != 0 replays one CUDA graph of a whole step. */
int moloch_gpu_run(moloch_handle_t* h, int nsteps, int use_graph);

/* Copy a field back into a reference-layout host array. */
int moloch_gpu_download(moloch_handle_t* h, int field, double* host_base,
                        const int* lb, const int* ub);

/* How moloch_gpu_upload moves prognostic fields from the caller's host
 * arrays to the device.  Direct (1): a kernel reads the host array itself
 * through the host page tables (NVLink-C2C on GB300, about 185 GB/s: 0.7 ms
 * for a 512x512x60 FP64 field against 1.8 ms staged), gathering the
 * interior and converting to the bulk type on the device; the upload
 * returns once the kernel is done.  Staged (0): host threads convert level
 * chunks into pinned staging that cudaMemcpyAsync moves.  Direct is the
 * default where the device reports pageable memory access with host page
 * tables.  Uploads from ranges registered with moloch_gpu_host_register
 * are DMA copies in either mode.  Downloads and the output path are always
 * staged (a kernel
 * writing into host pages not yet touched takes a page fault per page).
 * enable: 1 use direct when supported, 0 staged, -1 only query.  Returns
 * the mode in effect (0 or 1) or a negative error. */
int moloch_gpu_host_direct(moloch_handle_t* h, int enable);

/* Register (pin, cudaHostRegister) a host range whose arrays will be
 * uploaded again and again -- a Fortran driver's module arrays, allocated
 * once.  An upload from inside a registered range is a copy-engine DMA of
 * the whole Fortran array into a device staging buffer on the handle's
 * upload stream, overlapping the steps already issued without taking SMs;
 * a gather/convert kernel on the step stream then commits it in stream
 * order.  The call returns once the DMA is done.  The range must stay
 * allocated until moloch_gpu_host_unregister (or moloch_gpu_destroy). */
int moloch_gpu_host_register(moloch_handle_t* h, const void* ptr, size_t bytes);
int moloch_gpu_host_unregister(moloch_handle_t* h, const void* ptr);

/* Output path (nompi/regcm_dynamical_core.F90:203-216 writes t and ps
 * every iout steps).  output_start snapshots t and ps on the device in
 * stream order (after the steps already issued) and starts their copy to
 * pinned host memory on a second stream, then returns: the next steps run
 * while the copy is in flight.  output_finish waits for that copy and fills
 * reference-layout host arrays (either may be NULL) with the snapshot.
 * When both given arrays lie in ranges registered with
 * moloch_gpu_host_register, a kernel on the second stream lays the
 * snapshot out in their Fortran order on the device and the copy engine
 * writes them, instead of host threads. 
 * One snapshot at a time: start, finish, start, ... */
int moloch_gpu_output_start(moloch_handle_t* h);
int moloch_gpu_output_finish(moloch_handle_t* h, double* t_host, const int* t_lb, const int* t_ub,
                             double* ps_host, const int* ps_lb, const int* ps_ub);

/* Block until the handle's stream is idle.  MOLOCH_ERR_TIMEOUT when a
 * bounded wait of the staged column kernel gave up since the last check
 * (the state is then invalid); lprint steps check the same flag. */
int moloch_gpu_sync(moloch_handle_t* h);

/* Bounded device waits of the staged column kernel (tuning bit 32): every
 * wait gives up after `cycles` SM clock cycles (<= 0: the default, 2e9,
 * about one second), sets the flag moloch_gpu_sync reports and lets the
 * kernel return.  skip_job >= 0 is a test hook: the kernel's loader leaves
 * that staged chunk (counted per CTA from 0) unissued, so a wait on it
 * runs out; -1 turns it off.  No reference counterpart (the reference has
 * no device waits). */
int moloch_gpu_set_wait_limit(moloch_handle_t* h, long long cycles, int skip_job);

/* Arithmetic check (tests): for n device values, q_corr = the quotient the
 * FP32 Exner/theta update uses (reciprocal estimate with one residual
 * correction) and q_ieee = CUDA's IEEE FP32 quotient a / b, on the given
 * stream (a cudaStream_t, NULL for the default).  No reference
 * counterpart. */
int moloch_gpu_check_division(const float* a, const float* b, float* q_corr, float* q_ieee, int n, void* stream);

/* The same for FP64 (tests): q_nr = the quotient the contracting build's
 * WAF limiter uses (FP32 reciprocal estimate, two Newton-Raphson steps, one
 * residual correction) and q_ieee = CUDA's IEEE FP64 quotient.  No
 * reference counterpart. */
int moloch_gpu_check_division_f64(const double* a, const double* b, double* q_nr, double* q_ieee, int n,
                                  void* stream);

/* The stream the handle launches on (a cudaStream_t). */
void* moloch_gpu_stream(moloch_handle_t* h);

/* Number of kernels this handle has launched (graph replays count each
 * kernel node), for launch accounting. */
long long moloch_gpu_kernel_count(moloch_handle_t* h);

/* Run one phase of the step, for per-phase parity checks:
 * 0 = reset_tendencies + pre-diagnostics (:289-323), 1 = sound() (:483-851),
 * 2 = advection() (:897-927), 3 = filters + post-diagnostics (:333-391). */
int moloch_gpu_phase(moloch_handle_t* h, int phase);

/* One step with a CUDA event before and after every kernel on the handle's
 * stream; adds the milliseconds of each kernel kind to ms_by_kind[kind]
 * (kinds 0 .. moloch_gpu_kernel_kinds()-1) and the launch counts to
 * launches_by_kind (either array may be NULL).  For profiling and the
 * roofline report; the reference only times the whole run
 * (nompi/regcm_dynamical_core.F90:30,222-228). */
int moloch_gpu_profile_step(moloch_handle_t* h, double* ms_by_kind, int* launches_by_kind, int nkinds);
int moloch_gpu_kernel_kinds(void);
const char* moloch_gpu_kernel_name(int kind);

/* Project-written autotuner.  Launch shapes that depend on the grid are
 * timed with CUDA events on the handle's stream and the fastest is kept
 * (moloch_gpu_tuning_count() slots):
 *   choice[0] = horizontal WAF kernel: 1, 2, 4, 8 levels per 32x8 tile
 *               block, or 16, 32, 64 rows per warp strip;
 *   choice[1] = sound kernel variants, bit mask: 1 divergence, 2 damping,
 *               4 momentum as k-marching kernels (chunks of 4 levels per
 *               thread, next level prefetched), 8 momentum as warp strips
 *               (30 columns x 32 rows), 16 divergence and damping fused in
 *               one warp-strip kernel (29 columns x 32 rows; overrides 1
 *               and 2), 32 the implicit-w column solve staged by TMA with
 *               its column state in TMEM (FP32 storage, jx a multiple of 4,
 *               kz <= 64; elsewhere the bit is ignored), 64 (with 8) the
 *               momentum strips with two columns per lane (62 columns x 32
 *               rows per warp, 8-byte copies; FP32 storage, jx even;
 *               elsewhere, and in ensembles, the one-column strips), 128
 *               or 256 (with 32) the staged column solve with two words of
 *               column state a level in TMEM and 12 or 16 compute warps
 *               per SM (the old w and zdiv2b staged again for the
 *               back-substitution; bit-identical to bit 32 alone; not both,
 *               and not in ensembles), 512 (with 16) the fused
 *               divergence/damping strips over two levels per warp
 *               (shared row loads; not in ensembles); 0 = one level per
 *               thread;
 *   choice[2] = advected fields per thread of the vertical WAF kernel:
 *               1, 2, 5 or 10 (the fields of a thread share the velocity
 *               loads and terms);
 *   choice[3] = rows per warp strip of the momentum strips, 4 to 64
 *               (candidates 4, 8, 16, 32: shorter strips put more warps in
 *               flight; in ensembles the one-launch-per-kernel mode takes
 *               it, the persistent kernel keeps 32);
 *   choice[4] = 1: the staggering back from the cross points with four
 *               columns per thread and 16-byte loads and stores (FP32
 *               storage, jx a multiple of 4; elsewhere, and in ensembles,
 *               ignored), 0: one column per thread.
 * moloch_gpu_autotune runs advection() and sound() once per candidate and
 * repeat, so it advances the model state: call it on a scratch handle or before the
 * initial state is uploaded again.  The chosen values can be cached by the
 * caller and applied to new handles with moloch_gpu_set_tuning, which
 * refuses an out-of-range slot with MOLOCH_ERR_ARG and then leaves every
 * slot as it was.  No reference counterpart (the reference has no GPU
 * launch shapes). */
int moloch_gpu_tuning_count(void);
int moloch_gpu_autotune(moloch_handle_t* h, int* choice, double* best_ms, int nchoice);
int moloch_gpu_set_tuning(moloch_handle_t* h, const int* choice, int nchoice);

/* ---- ensembles --------------------------------------------------------------
 * Many domains of uneven size (jx, iy, kz may all differ) advanced together,
 * one step of the whole ensemble as one CUDA graph, in one of two modes:
 *   - per kernel: each kernel of the step is ONE launch whose 1-D grid walks
 *     a table of (member, tile) entries over all members, heaviest column
 *     tiles first;
 *   - persistent (moloch_gpu_ensemble_set_persistent): the whole step is ONE
 *     cooperative launch of as many blocks as fit on the GPU at once, walking
 *     the kernels of the step as phases separated by grid barriers; within a
 *     phase blocks take (member, tile) items from a device-side work queue.
 *     Same kernel bodies, so the same results as the per-kernel mode.
 *     Barrier waits are bounded (moloch_gpu_ensemble_set_wait_limit); one that
 *     gives up abandons the step, and moloch_gpu_ensemble_sync reports it.  Members are ordinary
 * handles created by the caller on the same stream with the same mode,
 * mo_nadv, mo_nsound and filter switches (the theta/pai filters are not
 * supported in ensembles), each initialized (setup_idealized or uploads +
 * moloch_gpu_init).  After moloch_gpu_ensemble_run every member handle holds
 * its advanced state (download, lprint via moloch_gpu_step, etc. work as for
 * a single domain).  The reference runs one domain per process; these calls
 * have no reference counterpart. */
typedef struct moloch_ensemble moloch_ensemble_t;
int moloch_gpu_ensemble_create(int nmembers, moloch_handle_t* const* members, moloch_ensemble_t** out);
int moloch_gpu_ensemble_run(moloch_ensemble_t* e, int nsteps, int use_graph);
/* event-timed choice of the launch shapes over the whole ensemble (advances
 * the members' state); choice as for moloch_gpu_autotune */
int moloch_gpu_ensemble_autotune(moloch_ensemble_t* e, int* choice, double* best_ms, int nchoice);
int moloch_gpu_ensemble_set_tuning(moloch_ensemble_t* e, const int* choice, int nchoice);
long long moloch_gpu_ensemble_kernel_count(moloch_ensemble_t* e);
/* persistent mode: 0 off; 2, 3 or 4 on, with the kernel built for that many
 * resident blocks of 256 threads per SM (register budgets 128, 80, 64);
 * 1 on with the last build chosen (3 at first).  It carries the horizontal WAF as tiles
 * (choice[0] 1..8), 1 or 2 vertical-WAF fields per thread, the one-thread
 * column solve (no bit 32), and in FP32 no k-marching momentum (choice[1]
 * bit 4 without 8), in FP64 no fused divergence/damping strips (bit 16);
 * other tunings give MOLOCH_ERR_ARG.  In the one-launch-per-kernel mode an
 * ensemble takes choice[1] bits 1 to 32 and 512 (bit 32: the staged column
 * solve for its FP32 members with tensor maps; bit 512 with 16: the fused
 * strips over two levels per warp) and choice[3], the rows per momentum
 * strip.
 * moloch_gpu_ensemble_autotune times one launch per kernel and the three
 * builds on whole steps and keeps the fastest; moloch_gpu_ensemble_persistent
 * returns the blocks per SM of the build in use, 0 when the mode is off. */
int moloch_gpu_ensemble_set_persistent(moloch_ensemble_t* e, int on);
int moloch_gpu_ensemble_persistent(moloch_ensemble_t* e);
/* One ensemble step (not graph-captured) timed per kernel kind, in the
 * buckets of moloch_gpu_profile_step: per-kernel mode, CUDA events around
 * every launch; persistent mode, the GPU global timer read by block 0 as it
 * leaves each grid barrier (a phase's time includes its barrier).  Adds to
 * ms_by_kind / launches_by_kind (phases per kind in persistent mode). */
int moloch_gpu_ensemble_profile_step(moloch_ensemble_t* e, double* ms_by_kind, int* launches_by_kind, int nkinds);
/* Limit of every grid-barrier wait of the persistent kernel, in SM clock
 * cycles (<= 0: the default 2e9, about one second).  skip_block/skip_barrier
 * (-1: off) are a test hook: that block leaves the launch at that barrier
 * without arriving, so the other blocks' waits run out. */
int moloch_gpu_ensemble_set_wait_limit(moloch_ensemble_t* e, long long cycles, int skip_block, int skip_barrier);
/* Block until the ensemble's stream is idle.  MOLOCH_ERR_TIMEOUT when a
 * barrier wait of the persistent kernel gave up since the last sync (those
 * steps, and the ones after them up to this call, did not complete; the
 * flag is cleared, so later steps run again). */
int moloch_gpu_ensemble_sync(moloch_ensemble_t* e);
int moloch_gpu_ensemble_destroy(moloch_ensemble_t* e);

/* ---- tensor-core GEMM (tcgen05) used by the acoustic-cycle surrogate --------
 * C = act(A * B^T + bias) on device buffers: A [M][K] and B [N][K] BF16
 * row-major (K contiguous), C [M][N] FP32 (ldc) and/or Cb BF16 (ldcb, holds
 * act(...)); act 0 = identity, 1 = SiLU; bias may be NULL.  Requires
 * N % 16 == 0, K % 64 == 0 and 16-byte aligned rows.  Accumulation is FP32
 * in tensor memory.  No reference counterpart. */
int moloch_tc_gemm(const void* A, int lda, const void* B, int ldb, float* C, int ldc, void* Cb, int ldcb,
                   const float* bias, int M, int N, int K, int act, void* stream);
/* MOLOCH_ERR_TIMEOUT if a bounded tensor-core wait gave up since the last
 * call (synchronises the device and clears the flag), else MOLOCH_OK. */
int moloch_tc_status(void);
/* Limit of every mbarrier wait of the GEMM kernel (loader, MMA issuer,
 * epilogue, final drain), in SM clock cycles (<= 0: the default 2e9, about
 * one second); a wait that runs out sets the flag moloch_tc_status reads,
 * and the kernel drains its loads in flight and frees its tensor memory
 * before it returns.  skip_cta / skip_chunk (-1: off) are a test hook: that
 * CTA's loader leaves that K chunk (counted over the CTA's tiles) unarmed
 * and unissued, so the MMA wait for it runs out.  Process-wide settings. */
int moloch_tc_set_wait_limit(long long cycles, int skip_cta, int skip_chunk);

/* ---- learned acoustic-cycle surrogate ---------------------------------------
 * A per-column MLP that replaces one sound() call (the mo_nsound acoustic
 * substeps, nompi/mod_moloch.F90:483-851) on FP32-storage handles.  Input:
 * u, v, w (levels 2..kz+1), pai, tetav of the column and its 8 neighbours
 * (45*kz features, normalised per field and level); output: the increments
 * of the same five fields of the centre column over the whole cycle.
 * Layers: 45kz -> 256 -> 256 -> 256 -> 5kz, SiLU, BF16 operands and FP32
 * accumulation on tcgen05 for training and inference.  No reference
 * counterpart.
 * While attached, each sound() call first runs the MLP over every column.
 * Its increments are committed (and the plain substeps return at once)
 * when all of these hold, else the plain sound loop runs unchanged:
 *   - every increment is finite and |normalised| <= threshold x the largest
 *     |normalised target| of that output in the training set (x 1 before
 *     moloch_sur_prepare);
 *   - the cycle is not a judge cycle: every judge_every-th call (the first
 *     included; 0 = never) runs the plain loop, which judges the
 *     prediction of that cycle;
 *   - the last judge found the relative RMS error of the increments (worst
 *     of the five fields) <= tol (with judge_every == 0 it is never judged
 *     and starts enabled).
 * All decisions are taken on the device, so a step stays one graph.
 *   create:   kz, dataset capacity (pairs), batch rows (multiple of 64)
 *   collect:  advance the handle nsteps plain steps, recording
 *             cols_per_cycle random columns per sound() call as pairs
 *   prepare:  normalisation statistics, shuffle, validation split
 *   train:    iters Adam steps (cosine decay from lr); returns the mean
 *             squared error in normalised units on training rows and on
 *             the validation split
 *   attach:   s == NULL detaches; the surrogate must outlive the attachment
 *   counts:   counts4 = {sound() calls, calls run by the plain loop, judge
 *             calls, judge verdicts that disabled the surrogate}; the
 *             largest |y| / envelope since attach; the last judge's error
 *   param:    layer weights [out][in] and bias, read (set 0) or written
 *   gradients: one forward+backward pass on n == batch rows of normalised
 *             features X [n][kin] and targets T [n][nop]: summed squared
 *             error and one layer's gradients (for gradient checks)
 *   dims:     kz, nin, kin, nout, nop, hidden, batch, pairs, training rows
 *   stats:    the normalisation statistics */
typedef struct moloch_surrogate moloch_surrogate_t;
int moloch_sur_create(int kz, int capacity, int batch, unsigned long long seed, moloch_surrogate_t** out);
int moloch_sur_collect(moloch_surrogate_t* s, moloch_handle_t* h, int nsteps, int cols_per_cycle,
                       unsigned long long seed);
int moloch_sur_pairs(moloch_surrogate_t* s);
/* copy collected pairs first .. first+count-1 to the host: X [count][45*kz]
 * raw FP32 features, T [count][5*kz] raw increments (output index
 * f*kz + k), in collection order (before moloch_sur_prepare shuffles its
 * normalised copies) */
int moloch_sur_pair_data(moloch_surrogate_t* s, int first, int count, float* X, float* T);
int moloch_sur_prepare(moloch_surrogate_t* s, double val_fraction, unsigned long long seed);
int moloch_sur_train(moloch_surrogate_t* s, int iters, float lr, unsigned long long seed, float* train_loss,
                     float* val_loss);
int moloch_sur_attach(moloch_handle_t* h, moloch_surrogate_t* s, float threshold, int judge_every, float tol);
int moloch_sur_counts(moloch_surrogate_t* s, long long* counts4, float* max_ratio, float* last_error);
int moloch_sur_param(moloch_surrogate_t* s, int layer, float* W, float* b, int set, int* in_out);
int moloch_sur_gradients(moloch_surrogate_t* s, const float* X, const float* T, int n, float* loss, int layer,
                         float* gW, float* gb);
int moloch_sur_dims(moloch_surrogate_t* s, int* dims);
/* CUDA-event times (ms) of the inference stages of one cycle on the
 * attached handle's current state: features, the four layers, the check
 * (nms >= 6).  Changes no field. */
int moloch_sur_profile(moloch_surrogate_t* s, moloch_handle_t* h, double* ms, int nms);
/* normalisation statistics, 5*kz each (field-major: u, v, w, pai, tetav):
 * read (set 0) or write (set != 0, which also makes the surrogate
 * attachable without moloch_sur_prepare) */
int moloch_sur_stats(moloch_surrogate_t* s, float* xmean, float* xstd, float* ymean, float* ystd, int set);
int moloch_sur_destroy(moloch_surrogate_t* s);

/* WAF advection of ONE field by dt_adv seconds (the arithmetic of wafone,
 * nompi/mod_moloch.F90:929-1311) that allocates no device memory.  It has
 * no counterpart in the reference: it exists for callers that own all
 * device memory themselves -- a Fortran model keeping its arrays in its own
 * CUDA/OpenACC data regions, or a framework with its own memory pool -- and
 * cannot let a library call cudaMalloc, which may synchronise the device,
 * grow past the caller's pool, or fail once the caller has reserved the
 * GPU's memory.  The caller passes device pointers in this library's dense
 * layout (j fastest, then i, then k; s and fmzf have kz+1 levels; msfu,
 * msfv, msfx are jx*iy periodic arrays) and pp is advected in place.
 * The two work arrays live in one fixed __device__ array of 32 MiB that
 * every GPU loading the library keeps until exit, so jx*iy*kz may not
 * exceed 2097152 (2^21) points and kz may not exceed 65535; larger sizes
 * return MOLOCH_ERR_ARG.  The first call on a device looks that array's
 * address up once (cudaGetSymbolAddress with the device current); under
 * CUDA's default lazy module loading that is also when the CUDA runtime
 * loads this code on the device and reserves the 32 MiB.  So make the
 * first call on each device before any stream capture and before the
 * program reserves the rest of the GPU's memory (its pool or data
 * regions); later calls reserve nothing.  All calls share the array, so
 * calls that overlap on the GPU (other streams, other threads) race; each
 * call overwrites the work arrays completely before reading them.  No
 * cudaMalloc, cudaFree or allocating library routine is called. */
int moloch_gpu_wafone_noalloc(double* pp, const double* s, const double* u, const double* v,
                              const double* fmz, const double* fmzf, const double* msfu,
                              const double* msfv, const double* msfx, int jx, int iy, int kz,
                              double dt_adv, double dx, double dzita, int rotllr, void* stream);

/* deallocate (the reference frees its pool at exit, memory_destroy). */
int moloch_gpu_destroy(moloch_handle_t* h);

/* Text of the last error raised on the calling thread ("" if none). */
const char* moloch_gpu_last_error(void);

/* ---- idealized initial state ---------------------------------------------
 * Host restatement of the reference driver's param() and init()
 * (nompi/regcm_dynamical_core.F90:93-201, nompi/mod_atmosphere.F90:171-235)
 * followed by the uploads and moloch_gpu_init(): the call sequence the
 * Fortran program performs before its time loop.  Additions that the
 * reference does not have: Gaussian hills in ht, a seeded theta noise
 * t += a*(2U-1)*pai on the lowest `pert_levels` levels (splitmix64 of the
 * linear index), and the background wind u0, v0 (reference: 1, 1). */
typedef struct moloch_ideal {
  int nhills;
  double hill_h[4], hill_j[4], hill_i[4], hill_r[4]; /* m, centre (grid points), e-folding radius */
  double pert_amp;
  int pert_levels;
  unsigned long long seed;
  double u0, v0;
} moloch_ideal_t;

int moloch_gpu_setup_idealized(moloch_handle_t* h, const moloch_ideal_t* ideal);

/* The same initial state computed on the device, one thread per column
 * (no host arrays of the grid size are built or uploaded): the prognostic
 * fields are written in place, the FP64 static fields are copied back to
 * the library's host copies, then moloch_gpu_init runs.  Results agree with
 * moloch_gpu_setup_idealized to the rounding of exp/pow/sqrt (CUDA's versus
 * the host library's). */
int moloch_gpu_setup_idealized_device(moloch_handle_t* h, const moloch_ideal_t* ideal);

#ifdef __cplusplus
}
#endif
#endif /* MOLOCH_GB300_H */
