/*
 * funwave_gpu.h -- C ABI of the GB300 (sm_103a) FUNWAVE-TVD solver stage.
 *
 * The reference (mayhl/FUNWAVE-TVD) has no plugin API: its hot path is a set
 * of argument-less Fortran subroutines called from the time loop of
 * src/main.F:284-535 on shared MODULE GLOBAL state (src/mod_global.F).  This
 * library replaces that loop body.  A Fortran host binds these functions with
 * ISO_C_BINDING (BIND(C) interfaces, VALUE for the scalars); every entry point takes plain pointers,
 * sizes and a POD parameter block, returns an int status (0 = OK, negative =
 * FW_ERR_*), never exits, aborts or traps, and keeps all solver state
 * resident on one GPU between calls.
 *
 * Host arrays are Fortran column-major with the reference's extents and ghost
 * cells (Nghost = 3):  cell arrays Mloc x Nloc, x-face arrays (Mloc+1) x
 * Nloc, y-face arrays Mloc x (Nloc+1), Mloc = Mglob + 6, Nloc = Nglob + 6;
 * reals are double (REAL(SP) of the FP64 build), masks int32 (default
 * INTEGER).  The device layout is private.
 */
#ifndef FUNWAVE_GPU_H
#define FUNWAVE_GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define FW_OK               0
#define FW_ERR_CUDA        -1   /* a CUDA runtime call failed */
#define FW_ERR_OOM         -2   /* device allocation failed */
#define FW_ERR_BAD_PARAM   -3   /* invalid argument or parameter block */
#define FW_ERR_BLOWUP      -4   /* CHECK_BLOWUP: max|eta| > EtaBlowVal */
#define FW_ERR_NAN         -5   /* non-finite eta */
#define FW_ERR_UNSUPPORTED -6   /* option not built into this library */
#define FW_ERR_NOT_READY   -7   /* call order violated (e.g. step before init) */
#define FW_ERR_NO_DEVICE   -8   /* no usable CUDA device */
#define FW_ERR_IO          -9   /* checkpoint file unreadable, unwritable or malformed */
#define FW_ERR_TIMEOUT     -10  /* a bounded device wait ran out (the kernel gave up and returned) */

/* precision of the bulk arithmetic */
#define FW_PREC_FP64  0   /* every field and operation in double */
#define FW_PREC_MIXED 1   /* fields and fluxes in float; tridiagonal u/v
                             recovery and total-depth tests in double */

/* wavemaker kinds (WAVEMAKER key) */
#define FW_WK_NONE   0
#define FW_WK_REG    1    /* WK_REG   (wavemaker.F:67-194, 2369-2405) */
#define FW_WK_JON_2D 2    /* JON_2D   (wavemaker.F:370-413, 2128-2357) */

/* directional spreading of JON_2D */
#define FW_SPREAD_WRAPPED_NORMAL 0   /* the reference's Sigma_Theta form */
#define FW_SPREAD_COS2S          1   /* cos^2s((theta-theta_p)/2), s = spread_s */

/* Parameter block: the input.txt keys of the hot path with the reference's
 * names in the comments and defaults of src/io.F.  fw_params_default()
 * fills the defaults. */
typedef struct fw_params {
    int    Mglob, Nglob;          /* Mglob, Nglob */
    double DX, DY;                /* DX, DY */
    int    periodic;              /* PERIODIC          (F) */
    int    dispersion;            /* DISPERSION        (T) */
    double gamma1, gamma2, gamma3, beta_ref;  /* Gamma1..3 (1), Beta_ref (-0.531) */
    int    viscosity_breaking;    /* VISCOSITY_BREAKING (T) */
    int    show_breaking;         /* SHOW_BREAKING     (T) */
    double cbrk1, cbrk2;          /* Cbrk1 (0.65), Cbrk2 (0.35) */
    double wavemaker_cbrk;        /* WAVEMAKER_Cbrk    (1.0) */
    double nu_bkg;                /* nu_bkg            (0) */
    double swe_eta_dep;           /* SWE_ETA_DEP       (0.8) */
    double cfl;                   /* CFL               (0.5) */
    int    fixed_dt;              /* 1 when DT_fixed is given */
    double dt_fixed;              /* DT_fixed */
    double froude_cap;            /* FroudeCap         (3.0) */
    double min_depth;             /* MinDepth          (0.1) */
    double min_depth_frc;         /* MinDepthFrc       (0.1) */
    int    eta_limiter;           /* ETA_LIMITER       (F) */
    double trough_limit, crest_limit;  /* TroughLimit, CrestLimit */
    int    direct_sponge;         /* DIRECT_SPONGE     (F) */
    double sponge_west, sponge_east, sponge_south, sponge_north; /* Sponge_*_width (0) */
    double r_sponge, a_sponge;    /* R_sponge (0.85), A_sponge (5.0) */
    int    friction_sponge;       /* FRICTION_SPONGE   (F); CD_4_SPONGE uploaded */
    double cd_fixed;              /* Cd                (0) */
    int    wavemaker;             /* FW_WK_* */
    double amp_wk, tperiod, dep_wk, xc_wk, yc_wk, theta_wk, delta_wk; /* AMP_WK.. Delta_WK (0.5) */
    double time_ramp, ywidth_wk;  /* Time_ramp (0), Ywidth_WK (LARGE) */
    double freq_peak, freq_min, freq_max;      /* FreqPeak, FreqMin, FreqMax */
    double gamma_tma, hmo, theta_peak, sigma_theta; /* GammaTMA, Hmo, ThetaPeak, Sigma_Theta (10) */
    int    nfreq, ntheta;         /* Nfreq, Ntheta */
    int    spreading;             /* FW_SPREAD_* */
    double spread_s;              /* s of cos^2s */
    /* build-side options (not input.txt keys) */
    int    precision;             /* FW_PREC_FP64 or FW_PREC_MIXED */
    int    device;                /* CUDA device ordinal */
    int    track_hmax;            /* OUT_Hmax: keep the running max of eta */
    /* statistics (misc.F:307-383, mixing.F:53-305) */
    int    track_hmin, track_umax, track_mfmax;  /* OUT_Hmin, OUT_Umax, OUT_MFmax (F) */
    double steady_time;           /* STEADY_TIME (LARGE): time means and wave heights from then on */
    double t_intv_mean;           /* T_INTV_mean (LARGE): averaging interval */
    int    track_roller;          /* ROLLER or UNDERTOW output (F): BREAKING's ROLLER_FLUX, UNDERTOW_U/V */
    int    track_radiation;       /* Radiation, Umean or Vmean output (F): the radiation-stress, momentum-flux
                                     and breaking-dissipation sums of CALCULATE_MEAN (mixing.F:156-219) */
} fw_params;

typedef struct fw_ctx fw_ctx;

/* Fill p with the reference's input.txt defaults (src/io.F READ_* sites). */
void fw_params_default(fw_params *p);

/* Create a context and allocate its device state (no kernel runs yet).
 * Replaces ALLOCATE_VARIABLES (init.F:54-269) and INDEX (misc.F:54-178).
 * FW_ERR_UNSUPPORTED for a grid whose padded field plane, (Mglob+7 rounded
 * up to 32) x (Nglob+7) cells, would reach 2^31 elements (the kernels use
 * 32-bit offsets within a plane); FW_ERR_OOM when the state does not fit. */
int fw_create(const fw_params *p, fw_ctx **out);
int fw_destroy(fw_ctx *ctx);

/* Host-side INITIALIZATION (init.F:280-1272): depth ghosts and face depths,
 * EtaBlowVal, Cd, wavemaker coefficients (WK_REG; JON_2D spectrum and the
 * band Cm/Sm of CALCULATE_Cm_Sm), the direct sponge, MASK/dry eta, H, HU,
 * HV, Ubar, Vbar, MASK9 and the wavemaker band, then uploads everything.
 *   depth  interior depth, Mglob x Nglob column-major (DEPTH_TYPE=DATA)
 *   eta,u,v  optional interior initial state (INI_UVZ), NULL for zero
 *   phases optional JON_2D phases phi1(kf,ktheta), Nfreq x Ntheta column-
 *          major; the reference draws them from rand(0)
 *          (wavemaker.F:2342-2352), so a caller supplies them. */
int fw_init(fw_ctx *ctx, const double *depth, const double *eta, const double *u,
            const double *v, const double *phases);

/* Whole-field transfer by reference name ("Eta","U","V","Ubar","Vbar","HU",
 * "HV","H","MASK","MASK9","Depth","Depthx","Depthy","P","Q","Fx","Fy","Gx",
 * "Gy","U4","V4","U1p","V1p","Udisp","Vdisp","ETAx","ETAy","ETAT","AGE",
 * "nu_break","SPONGE","Cd","CD_4_SPONGE","MASK_STRUC","Eta0","Ubar0",
 * "Vbar0","U0","V0","SourceX","SourceY","WaveMaker_Mass","HeightMax"; with
 * statistics on: "HeightMin","VelocityMax","MomentumFluxMax","ETAmean",
 * "Umean","Vmean","ETA2mean","SigWaveHeight","WaveHeightAve",
 * "WaveHeightRMS","Emax","Emin","Num_Zero_Up" (a count, as double)).
 * host points to a Fortran-ordered array of the field's full extent
 * (double, or int32 for MASK/MASK9/MASK_STRUC).  Synchronous. */
int fw_get_field(fw_ctx *ctx, const char *name, void *host);
int fw_set_field(fw_ctx *ctx, const char *name, const void *host);
/* The same with float host arrays, for a host built in single precision
 * (the reference's default build: REAL(SP) = 4-byte reals, mod_param.F:58-
 * 68), whose GLOBAL arrays are float.  Any field but the masks (which stay
 * int32 through fw_get_field/fw_set_field).  Values are rounded to nearest
 * float on the way out of the FP64 build and exact in the mixed build.
 * Initial inputs (fw_init) stay double: a single-precision host widens its
 * depth and initial state once at start-up. */
int fw_get_field_f32(fw_ctx *ctx, const char *name, float *host);
int fw_set_field_f32(fw_ctx *ctx, const char *name, const float *host);
/* n fields at once (n <= 16, names as above, no masks) to or from float
 * host arrays, synchronous.  In a mixed context each field moves with one
 * 2-D copy straight between the host array and the device field (with
 * pinned host buffers, at the host link's rate, half the bytes of the
 * double transfers); an FP64 context converts field by field. */
int fw_set_fields_f32(fw_ctx *ctx, int n, const char *const *names, const float *const *host);
int fw_get_fields_f32(fw_ctx *ctx, int n, const char *const *names, float *const *host);
/* n fields at once (n <= 16; names and host layouts as above), synchronous.
 * fw_set_fields copies every plane to the device on a second stream and
 * converts each one as soon as it has arrived; fw_get_fields is
 * fw_output_begin followed by fw_output_wait.  With pinned host buffers
 * (fw_host_alloc) the copies run at the host link's rate. */
int fw_set_fields(fw_ctx *ctx, int n, const char *const *names, const void *const *host);
int fw_get_fields(fw_ctx *ctx, int n, const char *const *names, void *const *host);
/* The values of one field (names as fw_get_field) at n cells given by
 * 1-based Fortran indices I[k], J[k] (ghost cells included in the range),
 * as double (masks as 0/1).  For station output (STATIONS, io.F:3786-3954)
 * without moving whole fields.  Synchronous. */
int fw_get_points(fw_ctx *ctx, const char *name, int n, const int *I, const int *J, double *out);
/* scalars "TIME","DT","EtaBlowVal","T_brk","Width_WK","ilo","ihi","jlo","jhi","T_sum",
 * "ICOUNT_MEAN" (CALCULATE_MEAN intervals ended so far, the number of
 * PREVIEW_MEAN's files).  With track_radiation, fw_get_field also knows
 * CALCULATE_MEAN's "P_center","Q_center","U_davg","V_davg","Wsurf",
 * "BreakSourceX","BreakSourceY" (last stage's values), their sums
 * ("U_davg_sum" .. "BreakDissY_sum"), the means "U_davg_mean","V_davg_mean",
 * "P_mean","Q_mean","UUmean","UVmean","VVmean","WWmean","FRCXmean",
 * "FRCYmean","BreakDissX","BreakDissY" and the gradient fields "DxSxx",
 * "DySxy","DySyy","DxSxy","PgrdX","PgrdY","DxUUH","DyUVH","DyVVH","DxUVH"
 * (mixing.F:156-219).
 * "WAIT_LIMIT" (get and set) is not a reference quantity: the polls of the
 * bounded wait with which a TMA-staged flux tile waits for its copies
 * (0 = the default, about 0.3-1 s).  A wait that runs out leaves the
 * block's fluxes NaN, and the step reports FW_ERR_NAN; the context stays
 * usable.  Lowering it makes that path run on purpose (a test of failure
 * reporting).  Setting it drops the captured step graphs.
 * "BREAK_PASSES" (get and set) is not a reference quantity either: the
 * parallel passes of BREAKING's candidate sweep (breaker.F:182-224) before
 * the rest runs in one pass ordered by level i + 2j (default 8; 0 = the
 * level-ordered pass only).  Every value gives the sweep's result; it only
 * moves the time.  Setting it drops the captured step graphs. */
int fw_get_scalar(fw_ctx *ctx, const char *name, double *value);
int fw_set_scalar(fw_ctx *ctx, const char *name, double value);

/* --- time stepping (main.F:284-535) ------------------------------------ */
/* Eta0/Ubar0/Vbar0 copies, EXCHANGE, ESTIMATE_DT (TIME += DT), U0/V0
 * copies: main.F:295-331.  DT and TIME stay on the device. */
int fw_begin_step(fw_ctx *ctx);
/* One SSP-RK stage, istage = 1..3: main.F:382-485. */
int fw_stage(fw_ctx *ctx, int istage);
/* MIXING_STUFF (time means from STEADY_TIME on), MAX_MIN_PROPERTY and
 * CHECK_BLOWUP: main.F:496-517. *status gets FW_OK, FW_ERR_BLOWUP or
 * FW_ERR_NAN. */
int fw_end_step(fw_ctx *ctx, int *status);
/* nsteps whole steps (fw_begin_step + 3 fw_stage + fw_end_step), replayed
 * from a CUDA graph; *status as fw_end_step for the last step, checked
 * once at the end. */
int fw_step(fw_ctx *ctx, int nsteps, int *status);
/* fw_step split in two: enqueue nsteps whole steps on the context's stream
 * and return at once; then wait for them and get the CHECK_BLOWUP status of
 * those steps.  No reference counterpart (the reference steps one run). */
int fw_step_async(fw_ctx *ctx, int nsteps);
int fw_step_wait(fw_ctx *ctx, int *status);
/* An ensemble of independent runs (contexts of any sizes and precisions on
 * the same device): nsteps whole steps of each, enqueued round robin two
 * steps at a time so that the runs' streams execute concurrently, then
 * waited for; status[k] as fw_end_step for run k.  Each run's results are
 * those of fw_step on it alone, bit for bit.  No reference counterpart. */
int fw_ensemble_step(fw_ctx *const *ctxs, int n, int nsteps, int *status);
/* The same ensemble as one launch per two steps: fw_ensemble_create captures
 * every run's two-step graph as a child node of one parent CUDA graph (no
 * edges between runs, so they execute concurrently), and fw_ensemble_run
 * advances all runs by nsteps with one cudaGraphLaunch per two steps on the
 * ensemble's own stream (an odd last step is enqueued per run).  The parent
 * graph is rebuilt when a run's buffer state or launch shapes changed since
 * it was captured.  Work queued earlier on a run's stream completes first,
 * and work queued on it afterwards waits for the ensemble.  status[k] as in
 * fw_ensemble_step; results equal fw_step on each run alone, bit for bit.
 * The contexts must outlive the ensemble.  No reference counterpart. */
typedef struct fw_ensemble fw_ensemble;
int fw_ensemble_create(fw_ctx *const *ctxs, int n, fw_ensemble **out);
int fw_ensemble_run(fw_ensemble *ens, int nsteps, int *status);
int fw_ensemble_destroy(fw_ensemble *ens);
/* Synchronise the context's stream. */
int fw_sync(fw_ctx *ctx);

/* --- learned coarse-grid correction (no reference counterpart) ---------- */
/* A 4-layer 3x3 convolutional network on the coarse grid: inputs
 * (eta, u, v, depth / FW_NET_DEPTH_SCALE, MASK), three hidden layers of 32
 * channels with ReLU, outputs FW_NET_OUT_SCALE times the corrections of
 * (eta, u, v).  BF16 weights and activations, FP32 accumulation, FP32
 * master weights, gradients and Adam moments; zero padding at the edges.
 * Tensors are channels-last FP32 on the device: x [B][H][W][5], y and
 * targets [B][H][W][3], wmask [B][H][W], with W along the grid's x (I). */
#define FW_NET_DEPTH_SCALE 10.0
#define FW_NET_OUT_SCALE 100.0
typedef struct fw_net fw_net;
int fw_net_create(unsigned long long seed, fw_net **out);    /* He-initialised from seed */
int fw_net_destroy(fw_net *net);
long long fw_net_num_params(fw_net *net);
int fw_net_get_params(fw_net *net, float *host);            /* FP32 master weights, layer by layer: */
int fw_net_set_params(fw_net *net, const float *host);      /*   w[9][cin][cout] then b[cout] */
int fw_net_get_grads(fw_net *net, float *host);             /* gradients of the last fw_net_loss_grad */
int fw_net_forward(fw_net *net, const float *x, int B, int H, int W, float *y, void *stream);
/* forward, the masked mean squared error sum(wmask*(y-target)^2)/(B*H*W)
 * into *loss (host), and the gradients of every parameter */
int fw_net_loss_grad(fw_net *net, const float *x, const float *target, const float *wmask, int B, int H,
                     int W, double *loss, void *stream);
int fw_net_adam(fw_net *net, float lr, float beta1, float beta2, float eps, void *stream);
/* Polls of the tensor-core kernels' bounded waits (0 = the default, about
 * 0.3-1 s).  A wait that runs out makes the kernel give up, wait for its
 * own copies and MMAs, free its TMEM and return; the next call that reads
 * the status (fw_net_loss_grad with a loss pointer, fw_correct with
 * applied, fw_correct_run) returns FW_ERR_TIMEOUT and clears it.  Lowering
 * the limit makes that path run on purpose (a test of failure reporting). */
int fw_net_set_wait_limit(fw_net *net, unsigned polls);
/* Apply the network to a context's current state.  The correction acts on
 * the interior cells whose 3 x 3 neighbourhood is wet (MASK = 1 on the cell
 * and its eight neighbours; fw_net_set_shore_band changes the width), not
 * at the shoreline: the eta correction is projected to zero mean over those
 * cells (so the volume is unchanged), then eta, u, v (and H, HU, HV, Ubar,
 * Vbar to first order) are corrected there.  The plain step stands
 * (*applied = 0) when any |correction| exceeds max_corr, when a value is not
 * finite, when the raw eta correction's mean (the uniform rise or fall the
 * projection removes) exceeds max_corr / 2, or when a corrected total depth
 * would reach MinDepth.  The decision is made on the device: with applied
 * == NULL the call only enqueues work on the context's stream; with applied
 * given it waits and reports the decision. */
int fw_correct(fw_ctx *ctx, fw_net *net, double max_corr, int *applied);
/* The checks of the last fw_correct that was given applied: out[0] the raw
 * eta correction's mean, out[1] the cells it acts on, out[2] the largest
 * |correction| (m, m/s), out[3] the largest amount (m) by which a corrected
 * total depth would fall below MinDepth, out[4] 1 if applied else 0. */
int fw_net_last_check(fw_net *net, double *out);
/* The cells fw_correct acts on: those whose (2 cells + 1) x (2 cells + 1)
 * neighbourhood is wet; cells 0..3 (default 1; 0: every wet cell). */
int fw_net_set_shore_band(fw_net *net, int cells);
/* nsteps of (fw_step + fw_correct without waiting) on a coarse run, two
 * pairs per replay of one captured CUDA graph; status as fw_step's.  The
 * graph is captured again when the run, its buffer state, its launch
 * shapes or max_corr change; new weights are packed before each call.  No
 * reference counterpart. */
int fw_correct_run(fw_ctx *ctx, fw_net *net, int nsteps, double max_corr, int *status);

/* --- the reference's units, one call each (for coupling and parity) ---- */
int fw_exchange(fw_ctx *ctx);            /* EXCHANGE        bc.F:426 */
int fw_estimate_dt(fw_ctx *ctx);         /* ESTIMATE_DT     misc.F:216 */
int fw_cal_dispersion(fw_ctx *ctx);      /* CAL_DISPERSION  dispersion.F:62 */
int fw_fluxes(fw_ctx *ctx);              /* FLUXES          fluxes.F:52 */
int fw_source_terms(fw_ctx *ctx);        /* SourceTerms     sources.F:56 (materialises SourceX/Y) */
int fw_estimate_huv(fw_ctx *ctx, int istage); /* ESTIMATE_HUV etauv_solver.F:53 */
int fw_update_mask(fw_ctx *ctx);         /* UPDATE_MASK     masks.F:51 */
int fw_wave_breaking(fw_ctx *ctx);       /* WAVE_BREAKING   breaker.F:60 */
int fw_sponge_damping(fw_ctx *ctx);      /* SPONGE_DAMPING  sponge.F:52 */

/* Kernel launches issued by this context since creation (diagnostics;
 * launches recorded into a CUDA graph are counted once, at capture). */
/* Checkpoint / restore of the complete run state: every device field and
 * scalar the step reads (TIME, DT, masks, AGE, the statistics and their
 * compensation terms, the factorisation), the JON_2D band tables and the
 * values fw_init computed on the host.  A restored run continues bit for
 * bit as the checkpointed one.  Replaces the reference's HOT_START restart
 * from output fields (mod_global.F:387, io.F:805, main.F:189), which
 * restarts from rounded fields and zero statistics instead.
 *   fw_checkpoint  waits for the stream, then writes path; FW_ERR_IO when
 *                  the file cannot be written.
 *   fw_restore     into a context created with the same fw_params (device
 *                  may differ), initialised or not; FW_ERR_BAD_PARAM when
 *                  the parameters differ, FW_ERR_IO for an unreadable or
 *                  malformed file.  A failure after the file's header
 *                  checked out leaves the context un-initialised. */
int fw_checkpoint(fw_ctx *ctx, const char *path);
int fw_restore(fw_ctx *ctx, const char *path);

/* Asynchronous output: PREVIEW's field transfers (io.F:4304-4621) without
 * holding the time loop.
 *   fw_output_begin  enqueues on the context's stream a snapshot of n fields
 *                    (names as fw_get_field) into a device output buffer,
 *                    then their device-to-host copies into host[k] (the
 *                    layout and types of fw_get_field) on a second stream,
 *                    and returns without waiting.  The snapshot holds the
 *                    state after every step enqueued before the call; steps
 *                    enqueued after it run while the copies proceed.  A
 *                    call first waits for the previous call's copies.
 *                    host[k] must stay untouched until the copies are done
 *                    and should be pinned (fw_host_alloc) for them to
 *                    overlap with the steps.  FW_ERR_BAD_PARAM for an
 *                    unknown or switched-off field, before anything runs.
 *   fw_output_wait   waits for the copies of the last fw_output_begin.
 *   fw_output_done   1 when they are done (or none are pending), 0 while
 *                    they run, a negative status on an error; no wait.
 *   fw_host_alloc / fw_host_free  pinned host memory for the buffers. */
int fw_output_begin(fw_ctx *ctx, int n, const char *const *names, void *const *host);
int fw_output_wait(fw_ctx *ctx);
int fw_output_done(fw_ctx *ctx);
int fw_host_alloc(size_t bytes, void **ptr);
int fw_host_free(void *ptr);

long long fw_launch_count(fw_ctx *ctx);
/* Time nrep back-to-back launches of one kernel of the step with CUDA events
 * on the context stream; *ms_per_launch = average duration.  Names:
 * "disp_a","disp_b","flux_x","flux_y","update","tri_x","tri_y","post",
 * "mask","break_a","ghost","maskmul","begin".  Kernels that update state in
 * place (update, post, mask, maskmul, begin) change the state: time them on
 * a context whose state is disposable.  No reference counterpart. */
int fw_time_kernel(fw_ctx *ctx, const char *name, int nrep, double *ms_per_launch);
/* CUDA stream of the context, as a void* (cudaStream_t). */
void *fw_stream(fw_ctx *ctx);

/* --- launch-shape autotuning (no reference counterpart) ----------------- */
/* The tuning vector: FW_TUNE_LEN ints, (bx, by) thread-block shapes of the
 * per-cell kernels disp_a, disp_b, update, post_mask_break and maskmul
 * (bx a multiple of 32, bx*by <= 256), then the tile heights of the x-face
 * and the y-face flux kernels (8, 16 or 32 in MIXED; 8 or 16 in FP64), then
 * how those two stage their tiles (0: each thread loads its inputs; 1: TMA
 * tensor loads of the tile's fields into shared memory).  Every choice computes the same values bit for bit; only the speed
 * differs.  Defaults: 32 x 8 blocks, flux tiles 8 and 32 (16 in FP64). */
#define FW_TUNE_LEN 14
#define FW_TUNE_FRESH 1   /* fw_autotune flag: measure even if this shape was tuned before */
/* Choose the tuning vector by timing every candidate of each kernel on this
 * context's state with CUDA events (two sweeps, the faster of each), keeping
 * the fastest.  The state is saved to a temporary device copy first and put
 * back afterwards, so the run continues unchanged (the call allocates and
 * frees that copy: one arena's size).  Results are cached per process by
 * precision, size class (grids whose sides lie within the same powers of
 * two) and path, so an ensemble of many sizes tunes once per class.  Call
 * after fw_init; the next step recaptures its graph. */
int fw_autotune(fw_ctx *ctx, int flags);
int fw_get_tuning(fw_ctx *ctx, int *tuning);        /* FW_TUNE_LEN ints */
/* Set the tuning vector explicitly; FW_ERR_BAD_PARAM for a shape outside the
 * candidates above. */
int fw_set_tuning(fw_ctx *ctx, const int *tuning);

/* --- no device allocation ---------------------------------------------- */
/* The CFL time step of a grid whose velocity and depth arrays the caller
 * already holds on the GPU, computed without allocating any device memory:
 * for callers that cannot call cudaMalloc (device arrays owned by an OpenACC
 * or CUDA Fortran runtime, a fixed memory pool, a loop in which allocation
 * is forbidden).  It has no counterpart in the reference as an entry point.
 *   Mloc, Nloc the array extents (every cell, ghost cells included, takes
 *              part in the minimum)
 *   DX, DY     grid spacings (> 0)
 *   U, V, H    device pointers to contiguous Mloc x Nloc column-major double
 *              arrays of the velocities and the total depth, on the current
 *              CUDA device
 *   MinDepthFrc  floor of the depth in the wave celerity sqrt(g max(H, .))
 *   CFL        Courant number (> 0)
 *   dt_fixed   > 0: the step is dt_fixed halved until it is at most the CFL
 *              step; 0: the CFL step itself
 *   DT         device pointer, receives CFL * min(DX/(|U|+c), DY/(|V|+c))
 *              (or the halved dt_fixed)
 *   TIME       device pointer (or NULL), TIME += DT
 *   stream     cudaStream_t (NULL = legacy default stream)
 * Mloc*Nloc may be at most FW_DT_DEVICE_MAX_CELLS; larger grids get
 * FW_ERR_BAD_PARAM before anything runs, and so do pointers that are not
 * device (or managed) memory of the current device.  The call's scratch is
 * one static 512 KB device array per GPU: the first call in a CUDA context
 * looks up its address (set-up; make that first call before any stream
 * capture), and calls whose work overlaps on the GPU race on that array.
 * Asynchronous on stream; DT and TIME are valid once the stream reaches
 * that point. */
#define FW_DT_DEVICE_MAX_CELLS 134217728LL   /* 65536 blocks x 2048 cells */
int fw_estimate_dt_device(int Mloc, int Nloc, double DX, double DY, const double *U, const double *V,
                          const double *H, double MinDepthFrc, double CFL, double dt_fixed, double *DT,
                          double *TIME, void *stream);
/* Human-readable text of a status code. */
const char *fw_strerror(int status);

#ifdef __cplusplus
}
#endif
#endif
