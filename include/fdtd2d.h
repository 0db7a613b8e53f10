/*
 * fdtd2d.h -- C ABI of the GB300 TMz FDTD time-step engine.
 *
 * This header is the drop-in boundary for the reference's device driver
 * (FDTD_2D_Full/kernel.cu + Kernel.cuh).  The reference crosses that boundary
 * through implicit globals (FDTD_2D_Full/Ext_kernel.cuh:8-258) and four calls:
 *
 *   cudaError_t DevMemoryAllocation()     FDTD_2D_Full/Kernel.cuh:100  -> fdtd2d_create
 *   cudaError_t DevFieldCalculation()     FDTD_2D_Full/Kernel.cuh:102  -> fdtd2d_run (+ read_*)
 *   cudaError_t DevSourceToDetect...()    FDTD_2D_Full/Kernel.cuh:101  -> two contexts (vacuum + medium)
 *   cudaError_t DevMemoryFree()           FDTD_2D_Full/Kernel.cuh:106  -> fdtd2d_destroy
 *
 * Here the data that the reference passes in globals travels in one plain
 * struct (fdtd2d_setup) with pointers and sizes only.  The library copies what
 * it needs; the caller keeps ownership of every host buffer.  No C++ types and
 * no exceptions cross this ABI.  Every entry point returns 0 on success or a
 * negative FDTD2D_ERR_* code; fdtd2d_strerror() names it.
 *
 * Conventions shared with the reference (FDTD_2D_Full/kernel.cu:127-805):
 *   - Ez lives on an nx x ny grid (Imax x Jmax), x (index i) fastest.
 *   - Host-visible field layouts are the reference's own:
 *       Ez, Jz : [ny][nx]        Hx : [ny-1][nx]        Hy : [ny][nx-1]
 *   - Steps are numbered from 1 like the reference loop `for(n=1;n<=nMax;++n)`
 *     (FDTD_2D_Full/kernel.cu:2065).
 *   - One step = Hx, Hy (+CPML psi), Jz from Ez^n, Ez (+CPML psi), source,
 *     detectors -- the order of FDTD_2D_Full/kernel.cu:2073-2157.
 */
#ifndef FDTD2D_H
#define FDTD2D_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FDTD2D_ABI_VERSION 2

/* ---- status codes -------------------------------------------------------- */
enum {
    FDTD2D_OK            = 0,
    FDTD2D_ERR_INVALID   = -1,  /* bad argument or inconsistent setup          */
    FDTD2D_ERR_NOMEM     = -2,  /* device or host allocation failed            */
    FDTD2D_ERR_CUDA      = -3,  /* CUDA runtime error (fdtd2d_last_cuda_error) */
    FDTD2D_ERR_NONFINITE = -4,  /* NaN/Inf found in the fields                 */
    FDTD2D_ERR_RANGE     = -5,  /* step or index range outside the run         */
    FDTD2D_ERR_IO        = -6,  /* file could not be opened or written         */
    FDTD2D_ERR_CONFIG    = -7,  /* Settings.ini missing or malformed           */
    FDTD2D_ERR_STATE     = -8,  /* call not valid in the object's state        */
    FDTD2D_ERR_BUDGET    = -9,  /* request does not fit the HBM budget         */
    FDTD2D_ERR_NODEVICE  = -10, /* no CUDA device                              */
    FDTD2D_ERR_TIMEOUT   = -11  /* a bounded device-side wait gave up          */
};

/* ---- enumerations -------------------------------------------------------- */
enum { FDTD2D_MEDIUM_UNIFORM = 0,      /* scalar CA/CB/DA/DB + per-cell density map */
       FDTD2D_MEDIUM_MATERIAL_ID = 1 };/* ID1/ID2/ID3 maps + material tables        */

enum { FDTD2D_STORE_F32 = 0,           /* FP32 field storage (reference)            */
       FDTD2D_STORE_F16 = 1,           /* FP16 storage, per-array 2^k scale          */
       FDTD2D_STORE_BF16 = 2 };        /* BF16 storage                               */

enum { FDTD2D_FIELD_EZ = 0, FDTD2D_FIELD_HX = 1, FDTD2D_FIELD_HY = 2, FDTD2D_FIELD_JZ = 3,
       /* CPML auxiliary arrays in the reference's layouts (FDTD_2D_Full/kernel.cu:1160-1220) */
       FDTD2D_FIELD_PSI_EZX_1 = 4, FDTD2D_FIELD_PSI_EZX_2 = 5,   /* [ny][P]     */
       FDTD2D_FIELD_PSI_EZY_1 = 6, FDTD2D_FIELD_PSI_EZY_2 = 7,   /* [P][nx]     */
       FDTD2D_FIELD_PSI_HYX_1 = 8, FDTD2D_FIELD_PSI_HYX_2 = 9,   /* [ny][P-1]   */
       FDTD2D_FIELD_PSI_HXY_1 = 10, FDTD2D_FIELD_PSI_HXY_2 = 11  /* [P-1][nx]   */ };

typedef struct fdtd2d_point { int32_t i, j; } fdtd2d_point;

/*
 * Everything one shot needs; replaces the globals of FDTD_2D_Full/Ext_kernel.cuh.
 * Table index order is the reference's (index 0 = outer edge of each strip).
 */
typedef struct fdtd2d_setup {
    int32_t nx, ny;          /* Imax, Jmax                                        */
    int32_t npml;            /* PML_SIZE (FDTD_2D_Full/Settings.cuh:23); 2 <= P    */
    int32_t n_steps;         /* nMax                                              */
    double  dt, dx, dy;      /* s, m, m                                           */

    /* CPML recursion tables: E tables have npml entries, H tables npml-1
       (FDTD_2D_Full/FDTD_cuda.cu:1224-1460).                                     */
    const float *be_x_1, *ce_x_1, *be_x_2, *ce_x_2;
    const float *bh_x_1, *ch_x_1, *bh_x_2, *ch_x_2;
    const float *be_y_1, *ce_y_1, *be_y_2, *ce_y_2;
    const float *bh_y_1, *ch_y_1, *bh_y_2, *ch_y_2;
    /* update denominators 1/(kappa*d) (FDTD_2D_Full/FDTD_cuda.cu:1466-1578)      */
    const float *den_ex, *den_hx;           /* [nx-1] */
    const float *den_ey, *den_hy;           /* [ny-1] */

    /* medium */
    int32_t medium;                         /* FDTD2D_MEDIUM_*                     */
    float   ca, cb, da, db;                 /* uniform medium update coefficients  */
    const float *ne;                        /* uniform medium: [ny][nx] electron
                                               density at Ez cells (m^-3); NULL=none */
    const int32_t *id1, *id2, *id3;         /* material medium: [ny][nx] maps for
                                               Hx, Hy, Ez (values 0..255)          */
    int32_t n_materials;                    /* material medium: table length <=256 */
    const float *mat_ca, *mat_cb, *mat_da, *mat_db, *mat_ne;
    double  nu;                             /* electron collision frequency, 1/s   */
    double  jz_coef;                        /* e^2/m_e used by the Jz update
                                               (reference D_CJ = 2.81794e-8,
                                               FDTD_2D_Full/kernel.cu:119)         */

    /* phased-array soft source: Ez(src_e) -= s_e(n) after the E update, with
       s_e(n) = src_scale*envelope[n]*cos(2*src_pi*(beta/2*t^2 + f0*t + phase_e/360)),
       t = n*dt, beta = (f1-f0)/t1  (FDTD_2D_Full/kernel.cu:621-659, 694-698)   */
    int32_t n_src;
    const fdtd2d_point *src;                /* [n_src] absolute Ez cells           */
    const double *src_phase_deg;            /* [n_src]                             */
    const float *envelope;                  /* [n_steps+1], index = step n         */
    double  src_scale;                      /* reference: 1/(qantI*qantK)          */
    double  f0, f1, t1;                     /* Hz, Hz, s (t1 > 0 when f1 != f0)    */
    double  src_pi;                         /* pi used in the phase (reference 3.14) */

    /* detectors (FDTD_2D_Full/kernel.cu:719-805)                                 */
    int32_t n_det;  const fdtd2d_point *det;   /* Ez samples (D_detect)           */
    int32_t n_comp; const fdtd2d_point *comp;  /* Ez/Hx/Hy samples (D_det_*)      */
    int32_t record_traces;                  /* keep per-step samples on the GPU    */
    double  dft_freq;                       /* running FP64 DFT of the Ez detector
                                               samples at this frequency (0 = off) */
    int32_t storage;                        /* FDTD2D_STORE_*                      */

    /* wave-front ("RC") tracker, Dev_RCcalc (FDTD_2D_Full/kernel.cu:968-1044).
       After each step n, for each line l:
         edge_l = max(edge_l, rc_level * max(Ez(rc_max_i[l], 0),
                                             max_{j in [rc_j_cut, ny-2)} Ez(rc_max_i[l], j)))
         spd[n][l] = largest j in [1, ny-3] with !(|Ez(rc_scan_i[l], j)| < edge_l), else 0
       with edge_l starting at rc_edge0 (reference 10.0).                         */
    int32_t n_rc;
    const int32_t *rc_scan_i, *rc_max_i;
    int32_t rc_j_cut;
    float   rc_level, rc_edge0;

    /* line probe for the time-of-flight post-processing (Dev_SaveLine,
       FDTD_2D_Full/kernel.cu:666-688): Ez(line_i0 .. line_i0+line_n-1, line_j)
       is kept for every step in [line_first, line_last].                        */
    int32_t line_n, line_i0, line_j, line_first, line_last;

    /* Launch coverage of the reference's eight update kernels, in launch
       order: Hx, Hx y-CPML, Hy, Hy x-CPML, Jz, Ez, Ez x-CPML, Ez y-CPML
       (FDTD_2D_Full/kernel.cu:2075-2121).  The reference sizes these grids with
       floor divisions (kernel.cu:2027-2033), so on small grids the threads with
       linear index l >= cover[k] do not exist and those cells are not updated.
       A cell update whose reference thread index is >= cover[k] is skipped
       here too; 0 means every cell is updated, a negative value none.
       Honoured by the material-ID medium (the Settings.ini path).             */
    int64_t cover[8];
    /* Reduced field storage (storage = F16 / BF16): expected peak |Ez| used to
       pick the per-array power-of-two scales (0 = estimated from the source
       amplitude, the array size, the carrier and the plasma drive).           */
    double  field_max;
} fdtd2d_setup;

/* ---- single shot (the reference's plain run) ------------------------------ */
typedef struct fdtd2d_ctx fdtd2d_ctx;

/* Allocate device state, upload tables/maps, zero the fields.
   Replaces DevMemoryAllocation (FDTD_2D_Full/kernel.cu:1087-1618). */
int fdtd2d_create(const fdtd2d_setup *setup, int device, fdtd2d_ctx **out);

/* Advance steps n_first..n_last inclusive (1-based).  n_first must be the step
   after the last one run.  Replaces the loop body of DevFieldCalculation
   (FDTD_2D_Full/kernel.cu:2065-2309).  Asynchronous; errors surface at the
   next synchronising call. */
int fdtd2d_run(fdtd2d_ctx *ctx, int32_t n_first, int32_t n_last);

/* Wait for queued work; returns FDTD2D_ERR_CUDA on a device-side failure. */
int fdtd2d_synchronize(fdtd2d_ctx *ctx);

/* Last completed-or-queued step number (0 before the first run). */
int fdtd2d_current_step(const fdtd2d_ctx *ctx, int32_t *n);

/* Copy per-step detector samples of steps n0..n1 (1-based) to caller buffers,
   row-major [n1-n0+1][n_det] (ez) and [n1-n0+1][n_comp] (comp_*).  Any pointer
   may be NULL.  Requires record_traces. */
int fdtd2d_read_traces(fdtd2d_ctx *ctx, int32_t n0, int32_t n1, float *det_ez,
                       float *comp_ez, float *comp_hx, float *comp_hy);

/* Wave-front positions spd[n][l] of steps n0..n1 into [n1-n0+1][n_rc]. */
int fdtd2d_read_rc(fdtd2d_ctx *ctx, int32_t n0, int32_t n1, int32_t *spd);

/* Line-probe samples of steps n0..n1 (inside [line_first, line_last]) into
   [n1-n0+1][line_n]. */
int fdtd2d_read_line(fdtd2d_ctx *ctx, int32_t n0, int32_t n1, float *out);

/* Running DFT X_e = sum_n Ez_e^n exp(-i 2 pi f n dt) per Ez detector. */
int fdtd2d_read_dft(fdtd2d_ctx *ctx, double *re, double *im);

/* Copy a field (FDTD2D_FIELD_*) in the reference layout to / from host memory. */
int fdtd2d_read_field(fdtd2d_ctx *ctx, int which, float *host);
int fdtd2d_write_field(fdtd2d_ctx *ctx, int which, const float *host);

/* Snapshot and restore of a shot's state after its last step, for preempting
   a long shot and resuming it later, here or in another process: the fields
   and CPML psi arrays (reference layouts), the FP64 DFT sums, the detector
   traces recorded so far, the wave-front tracker's and the line probe's
   state, and the step number.  fdtd2d_state_bytes gives the size of the host
   image; fdtd2d_save_state writes it (FDTD2D_ERR_RANGE if `bytes` is
   smaller); fdtd2d_load_state makes a context created from the same setup
   continue from it: its next run call starts at the saved step + 1 and gives
   the bits the shot would have given without the stop.  An image of another
   geometry, storage or detector set is FDTD2D_ERR_INVALID; a batch member is
   FDTD2D_ERR_STATE.  Both wait for the shot's queued work.  No counterpart in
   the reference (its field dumps, FDTD_2D_Full/kernel.cu:2173-2303, cannot
   be restarted from). */
int64_t fdtd2d_state_bytes(fdtd2d_ctx *ctx);
int fdtd2d_save_state(fdtd2d_ctx *ctx, void *buf, int64_t bytes);
int fdtd2d_load_state(fdtd2d_ctx *ctx, const void *buf, int64_t bytes);

/* Device-side scan for NaN/Inf in Ez/Hx/Hy/Jz; FDTD2D_ERR_NONFINITE if any. */
int fdtd2d_check_finite(fdtd2d_ctx *ctx);

/* Allocation-free non-finite scan of a caller-owned device array.
   No counterpart in the reference.  For callers that must not allocate GPU
   memory (a host program that owns all device memory through its own pool,
   or code whose latency budget cannot absorb a cudaMalloc/cudaFree): it
   counts the NaN/Inf values in d_data[0..n) using a fixed 16 KiB scratch
   array compiled into this library, so it calls no cudaMalloc or cudaFree.
   Returns FDTD2D_OK when all values are finite, FDTD2D_ERR_NONFINITE when
   some are not (count in *nonfinite if non-NULL), FDTD2D_ERR_RANGE when
   n > 2^31 (the scratch covers at most 2^31 values per call).  `stream` is a
   cudaStream_t (NULL = default stream) of the calling thread's current
   device, and d_data memory that device can read; the call waits for the
   stream.  The first call on a device (and the first after that device was
   reset) resolves the scratch address for it: make that call before
   capturing any stream into a CUDA graph.  All calls share the one scratch
   array, so calls whose GPU work overlaps race; serialise them. */
int fdtd2d_check_finite_noalloc(const float *d_data, int64_t n, int64_t *nonfinite, void *stream);

/* Release everything.  Replaces DevMemoryFree (FDTD_2D_Full/kernel.cu:2820-2987). */
int fdtd2d_destroy(fdtd2d_ctx *ctx);

/* Bytes of device memory one shot of this setup holds. */
int64_t fdtd2d_device_bytes(const fdtd2d_setup *setup);

/* Kernel launches issued by this context so far (for launch accounting). */
int64_t fdtd2d_launch_count(const fdtd2d_ctx *ctx);

/* Name of the step kernel this context launches, with its launch shape
   (e.g. "step_tma_kernel<4,3>", "step_tmat2_kernel<4,2,2>+step_tma_kernel<2,2>",
   "step_persist_kernel<0>"; no counterpart in the reference). */
const char *fdtd2d_kernel_name(const fdtd2d_ctx *ctx);

/* ---- Batched and continuous stepping (no counterpart in the reference, which
   runs one shot per process with global state, FDTD_2D_Full/kernel.cu:1928-2818).
   A batch advances many uniform-medium shots (CPML <= 120 cells, no wave-front
   tracker or line probe) together: one persistent launch per time step, issued
   in blocks captured as CUDA graphs, each shot at its own step.  Shots can be
   admitted between fdtd2d_batch_run calls while others are in flight.  A shot
   of at least 2^21 cells (FDTD2D_BATCH_SOLO_CELLS overrides; 0 for none) is
   a solo member instead: a full single shot on its own streams with its own
   kernel choice (two steps per pass where that wins), stepped from the same
   run calls; its budget share counts that path's two extra field buffers.
   The batch's kernel steps FP32 fields, so a shot with F16 or BF16 storage
   is a solo member whatever its size.  At most 8 solo members step at a
   time, the oldest admitted first (FDTD2D_BATCH_SOLO_ACTIVE overrides).  A
   solo member admitted while the batch has device work in flight is not
   timed at create: it takes its class's stored kernel choice, else the
   default one. ---- */
typedef struct fdtd2d_batch fdtd2d_batch;

/* hbm_budget_bytes <= 0: 90 % of the device memory free now. */
int fdtd2d_batch_create(int device, int64_t hbm_budget_bytes, fdtd2d_batch **out);
/* Admit a shot (its device state is allocated and uploaded now; its step 1
   runs in the next step the batch issues).  FDTD2D_ERR_BUDGET when its
   fdtd2d_device_bytes would exceed the remaining budget. */
int fdtd2d_batch_add(fdtd2d_batch *b, const fdtd2d_setup *setup, int32_t *shot);
/* Issue n_steps more steps of every admitted, unfinished shot (asynchronous). */
int fdtd2d_batch_run(fdtd2d_batch *b, int32_t n_steps);
/* Wait for the issued steps; FDTD2D_ERR_TIMEOUT if a kernel wait ran out. */
int fdtd2d_batch_synchronize(fdtd2d_batch *b);
/* Steps issued for a shot (it is finished when this equals its n_steps). */
int32_t fdtd2d_batch_shot_step(const fdtd2d_batch *b, int32_t shot);
/* The shot's context, for fdtd2d_read_* (which wait for the batch's stream);
   fdtd2d_run on it returns FDTD2D_ERR_STATE. */
fdtd2d_ctx *fdtd2d_batch_shot(fdtd2d_batch *b, int32_t shot);
/* Free a shot's device memory and its slot. */
int fdtd2d_batch_remove(fdtd2d_batch *b, int32_t shot);
int64_t fdtd2d_batch_free_bytes(const fdtd2d_batch *b);
int64_t fdtd2d_batch_launch_count(const fdtd2d_batch *b);
const char *fdtd2d_batch_kernel_name(const fdtd2d_batch *b);
int fdtd2d_batch_destroy(fdtd2d_batch *b);

/* ---- Serving loop (no counterpart in the reference): shots are queued as they
   arrive, admitted in arrival order while they fit the budget, stepped together
   in blocks of block_steps launches, and retired as soon as the GPU has
   finished them (their DFT and Ez traces copied out, their memory released
   behind the queued kernels). ---- */
typedef struct fdtd2d_server fdtd2d_server;

int fdtd2d_server_create(int device, int64_t hbm_budget_bytes, int32_t block_steps, fdtd2d_server **out);
/* Queue a shot under the caller's tag.  The setup and the arrays it points to
   must stay valid until the shot is admitted (a later fdtd2d_server_step).
   FDTD2D_ERR_BUDGET if it could never fit the budget. */
int fdtd2d_server_submit(fdtd2d_server *s, const fdtd2d_setup *setup, int64_t tag);
/* One scheduling round: admit, retire finished shots, issue one block (at most
   two blocks run ahead of the GPU).  Returns the number of shots finished in
   this round (>= 0) or a negative status. */
int fdtd2d_server_step(fdtd2d_server *s);
/* Pop the oldest finished shot: returns 1 (0 if none); its tag, detector count,
   step count, DFT (re, im per detector, up to max_det) and Ez traces
   ([n_steps][n_det], up to max_trace floats) into caller buffers (may be null). */
int fdtd2d_server_pop(fdtd2d_server *s, int64_t *tag, int32_t *n_det, int32_t *n_steps, double *dft,
                      int32_t max_det, float *trace, int64_t max_trace);
int fdtd2d_server_counts(const fdtd2d_server *s, int32_t *queued, int32_t *running, int32_t *finished);
/* Cancel the shots submitted under `tag`, wherever they are: queued ones
   leave the queue, running ones stop being stepped and their device memory
   is released (behind the kernels already queued for them), finished ones
   not yet popped are dropped.  No result of a cancelled shot is popped.
   Returns the number of shots cancelled (0 if none had the tag). */
int fdtd2d_server_cancel(fdtd2d_server *s, int64_t tag);
fdtd2d_batch *fdtd2d_server_batch(fdtd2d_server *s);
int fdtd2d_server_destroy(fdtd2d_server *s);

/* Number of CUDA devices visible to this process (0 when none). */
int fdtd2d_device_count(void);

/* Run steps n_first..n_last like fdtd2d_run, bracketed by CUDA events on the
   context's stream; *elapsed_ms receives the device time of the whole range. */
int fdtd2d_run_timed(fdtd2d_ctx *ctx, int32_t n_first, int32_t n_last, float *elapsed_ms);

/* Event timing of the kernel that steps the interior of the grid, the one
   that sets the step time: the two-step tensor kernel when the context runs
   two steps per pass (its launches only), else the one-step tensor kernel,
   else the kernel that steps the whole grid.  on = 1 records a CUDA event
   pair on the shot stream around each of its launches from then on; on = 0
   stops and clears the totals.  fdtd2d_step_kernel_time reports the summed
   device time of the launches timed so far (*ms), their number (*launches),
   the cells one launch updates (*cells) and the time steps it advances them
   (*steps).  No counterpart in the reference. */
int fdtd2d_time_step_kernel(fdtd2d_ctx *ctx, int on);

/* Forget the kernel choices fdtd2d_create keeps per shot class (the next
   shot of every class is timed again).  The choices are also persisted in a
   JSON file keyed by the device's name, SM count and compute capability, the
   version of the timing method (entries of another version are timed again)
   and the shot class: $FDTD2D_TUNE_CACHE, else
   $XDG_CACHE_HOME/fdtd2d/kernel_choices.json, else
   $HOME/.cache/fdtd2d/kernel_choices.json (FDTD2D_TUNE_CACHE=0: memory
   only).  A process reads the file at the first shot of a device, so a shot
   of a class an earlier process timed skips the timing; clearing affects
   this process's memory only.  No counterpart in the reference. */
void fdtd2d_clear_kernel_choices(void);
/* How the kernel choices of this context's create were made: 0 timed at
   create (or forced by FDTD2D_* overrides), 1 a choice this process kept
   from an earlier shot of the class, 2 a choice read from the persisted
   file, 3 the default choice taken without timing (a batch's solo member
   admitted while the batch had work in flight).  No counterpart in the
   reference. */
int fdtd2d_kernel_choice_source(const fdtd2d_ctx *ctx);
int fdtd2d_step_kernel_time(fdtd2d_ctx *ctx, double *ms, int64_t *launches, int64_t *cells, int32_t *steps);

/* Stability number of the explicit update with the Drude current:
   (c dt)^2 (1/dx^2 + 1/dy^2) + (w_p,max dt / 2)^2, w_p,max from the largest
   plasma drive of the setup.  Above 1 the scheme grows without bound. */
double fdtd2d_stability(const fdtd2d_setup *setup);

const char *fdtd2d_strerror(int status);
int fdtd2d_last_cuda_error(const fdtd2d_ctx *ctx);   /* cudaError_t value */
int fdtd2d_abi_version(void);

/* ---- host-side setup precompute (the reference's L2 layer) ---------------- */
typedef struct fdtd2d_problem fdtd2d_problem;   /* owns the arrays its setup points to */

/* Parameterised shot (synthetic workloads): grid, CPML grading, plasma profile,
   phased array and detectors.  Units are SI; each field's meaning is given
   beside it. */
typedef struct fdtd2d_spec {
    int32_t nx, ny, npml, n_steps;
    double  dx, dy;
    double  courant;            /* dt = courant*dx/(c*sqrt(2)) when dt <= 0        */
    double  dt;
    /* CPML grading (FDTD_2D_Full/FDTD_cuda.cu:1206-1214 form)                     */
    double  cpml_m, cpml_ma;    /* polynomial orders (reference 3, 1)              */
    double  sigma_factor;       /* sigma_max = factor*0.8(m+1)/(eta0*d) (ref 0.75) */
    double  kappa_max, alpha_max;
    /* plasma density profile at Ez cells                                          */
    int32_t profile;            /* 0 none, 1 linear slab, 2 tanh, 3 tanh x (1+rms*g) */
    double  ne_peak;            /* slab: density at x_hi; tanh: 2x amplitude (n = ne_peak/2*(1+tanh)) */
    double  x_lo, x_hi;         /* slab extent (cells)                              */
    double  x_center, width;    /* tanh centre and width (cells)                    */
    double  grf_rms, grf_corr;  /* random-field rms and correlation length (cells)  */
    uint64_t seed;
    double  nu;                 /* collision frequency (1/s)                        */
    /* phased array: element e at (src_i + e*src_di, src_j + e*src_dj)             */
    int32_t n_elem, src_i, src_j, src_di, src_dj;
    double  freq;               /* carrier (Hz)                                     */
    double  steer_deg;          /* beam steering angle from the array normal        */
    double  amp;
    int32_t pulse;              /* 0 Gaussian (t0, width), 1 raised-cosine ramp then CW */
    double  pulse_width;        /* Gaussian 1/e half-width or ramp length (s)       */
    double  pulse_t0;           /* Gaussian centre (s); <=0 -> 4 widths             */
    /* detectors: element e at (det_i + e*det_di, det_j + e*det_dj)                */
    int32_t n_det, det_i, det_j, det_di, det_dj;
    int32_t record_traces;
    double  dft_freq;           /* 0 -> freq                                        */
    int32_t storage;            /* FDTD2D_STORE_*                                   */
    double  field_max;          /* expected peak |Ez| for reduced storage (0 = estimate) */
} fdtd2d_spec;

/* Fill a spec with the plain 512^2 workload defaults. */
void fdtd2d_spec_defaults(fdtd2d_spec *spec);

int fdtd2d_problem_from_spec(const fdtd2d_spec *spec, fdtd2d_problem **out);

/* Reference drop-in: read Settings.ini (same sections, keys and defaults as
   readINIparam, FDTD_2D_Full/FDTD_cuda.cu:27-176) and build the setup the
   reference builds (FDTD_2D_Full/FDTD_cuda.cu:305-382, 1122-1579, 2602-3655). */
int fdtd2d_problem_from_ini(const char *ini_path, fdtd2d_problem **out);

/* The SourceToDetect vacuum shot of a Settings.ini: the same setup with no
   medium, fluctuation or wall (ObjectsEnable = false).  Replaces the first pass
   of initlimits in that mode (FDTD_2D_Full/FDTD_cuda.cu:389-406) feeding
   DevSourceToDetectInfluenceCalc (FDTD_2D_Full/kernel.cu:1620-1926). */
int fdtd2d_problem_from_ini_vacuum(const char *ini_path, fdtd2d_problem **out);

const fdtd2d_setup *fdtd2d_problem_setup(const fdtd2d_problem *p);
void fdtd2d_problem_free(fdtd2d_problem *p);

/* Host post-processing of the drop-in driver, callable on its own.
   fdtd2d_write_rc_lines: wave-front rows spd[n][l] (n = 0..n_rows-1, row 0 =
   before step 1, as the reference's PspdLine) -> RC_Line.txt and
   TAU_Line.txt in out_dir (RClineFilterPostTime, CalculateRCfromPwrLines,
   CalculateTaufromPwrLines, FDTD_2D_Full/kernel.cu:3188-3270).
   fdtd2d_write_tof: saved Ez line field[t][i] (t < times, i <
   fdtd2d_tof_width(p): the Settings.ini SizeI in grid points, SizeI / ds,
   as the reference's proc_field[t][size_i]) -> the time-of-flight files
   (processing_core, FDTD_2D_Full/processing.cu:6-144).  field must hold
   times * fdtd2d_tof_width(p) floats.
   Both use the Settings.ini parameters the problem was built from.          */
int fdtd2d_write_rc_lines(const fdtd2d_problem *p, const int32_t *spd, int32_t n_rows,
                          const char *out_dir);
int fdtd2d_write_tof(const fdtd2d_problem *p, const float *field, int32_t times, const char *out_dir);
/* Row length fdtd2d_write_tof reads: 0 for a problem not built from a
   Settings.ini, or whose [Processing] line is empty. */
int32_t fdtd2d_tof_width(const fdtd2d_problem *p);

/* Whole reference program on top of this ABI: Settings.ini in, the reference's
   output files (Detect.txt, detAll.txt, detEz/Hx/Hy.txt, Ez.txt,
   FieldSaveDat.txt, SourceP.txt, iniLOG.txt, log.txt) out in out_dir.
   Replaces main -> initlimits (FDTD_2D_Full/FDTD_cuda.cu:20, 384-441). */
int fdtd2d_run_settings(const char *ini_path, const char *out_dir, int device);

#ifdef __cplusplus
}
#endif
#endif /* FDTD2D_H */
