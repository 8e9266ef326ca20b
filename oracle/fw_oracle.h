/*
 * fw_oracle.h -- CPU oracle for the FUNWAVE-TVD SSP-RK3 solver stage.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C, FP64 restatement of the
 * reference Fortran (mayhl/FUNWAVE-TVD, the src/ .F files, built with
 * -DDOUBLE_PRECISION -DCARTESIAN, serial) used by tests/, by the smoke check
 * and by the CPU-baseline leg of bench.py as the checker and the timed CPU
 * baseline.  It is never linked into or called by the product library.
 *
 * Parity status: the reference cannot be compiled here (no Fortran compiler),
 * and the reference ships no golden vectors or known-answer tests for this
 * path, so this restatement is "parity unpinned" against the reference
 * itself.  It is pinned by analytic invariants (lake at rest, y-mirror
 * symmetry, mass budget) and by hand-derived known-answer cases in tests/.
 *
 * Layout: every array is Fortran column-major with the reference's extents,
 * 1-based indices translated with I-1 / J-1:
 *   cell arrays    Mloc  x Nloc    (Mloc = Mglob + 6, Nloc = Nglob + 6)
 *   x-face arrays  Mloc1 x Nloc    (Mloc1 = Mloc + 1)
 *   y-face arrays  Mloc  x Nloc1   (Nloc1 = Nloc + 1)
 * Masks are int32 (Fortran default INTEGER).
 */
#ifndef FW_ORACLE_H
#define FW_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Run-time parameters: the input.txt keys of the hot path (io.F defaults). */
typedef struct {
    int    Mglob, Nglob;
    double DX, DY;
    int    periodic;            /* PERIODIC (F) */
    int    dispersion;          /* DISPERSION (T) */
    double gamma1, gamma2, gamma3, beta_ref;   /* 1, 1, 1, -0.531 */
    int    viscosity_breaking;  /* VISCOSITY_BREAKING (T) */
    int    show_breaking;       /* SHOW_BREAKING (T) */
    double cbrk1, cbrk2;        /* 0.65, 0.35 */
    double wavemaker_cbrk;      /* 1.0 */
    double nu_bkg;              /* 0.0 */
    double swe_eta_dep;        /* 0.8 */
    double cfl;                 /* 0.5 */
    int    fixed_dt;            /* DT_fixed given */
    double dt_fixed;
    double froude_cap;          /* 3.0 */
    double min_depth;           /* 0.1 */
    double min_depth_frc;       /* 0.1 */
    int    eta_limiter;         /* ETA_LIMITER (F) */
    double trough_limit, crest_limit;
    int    direct_sponge;       /* DIRECT_SPONGE (F) */
    double sponge_west, sponge_east, sponge_south, sponge_north;  /* 0 */
    double r_sponge, a_sponge;  /* 0.85, 5.0 */
    int    friction_sponge;     /* FRICTION_SPONGE (F): CD_4_SPONGE supplied */
    double cd_fixed;            /* Cd (0) */
    /* wavemaker: 0 none, 1 WK_REG, 2 JON_2D (band Cm/Sm supplied) */
    int    wavemaker;
    double amp_wk, tperiod, dep_wk, xc_wk, yc_wk, theta_wk, delta_wk;
    double time_ramp, ywidth_wk;
    /* JON_2D (wavemaker.F:370-413, 2128-2357) */
    double freq_peak, freq_min, freq_max;   /* FreqPeak, FreqMin, FreqMax */
    double gamma_tma, hmo, theta_peak, sigma_theta;  /* GammaTMA, Hmo, ThetaPeak, Sigma_Theta */
    int    nfreq, ntheta;       /* Nfreq, Ntheta */
    int    spreading;           /* 0: reference wrapped normal; 1: cos^2s (extension) */
    double spread_s;            /* s of cos^2s */
    /* statistics (misc.F:307-383, mixing.F:53-305) */
    int    track_hmax, track_hmin, track_umax, track_mfmax;  /* OUT_Hmax, OUT_Hmin, OUT_Umax, OUT_MFmax (F) */
    double steady_time;         /* STEADY_TIME (LARGE): time means from this time on */
    double t_intv_mean;         /* T_INTV_mean (LARGE): averaging interval */
} ofw_params;

typedef struct ofw_ctx ofw_ctx;

ofw_ctx *ofw_create(const ofw_params *p);
void     ofw_destroy(ofw_ctx *o);

/* Field access by name ("Eta", "U", "MASK", "Depthx", ...).  Returns a
 * pointer into the oracle's storage; *kind = 0 cell, 1 x-face, 2 y-face;
 * *is_int = 1 for int32 mask arrays.  NULL for an unknown name. */
void *ofw_field(ofw_ctx *o, const char *name, int *kind, int *is_int);
/* Scalars: "TIME","DT","T_brk","EtaBlowVal","D_gen","beta_gen","rlamda",
 * "Width_WK","ilo","ihi","jlo","jhi" (1-based band indices). */
double  ofw_get_scalar(ofw_ctx *o, const char *name);
void    ofw_set_scalar(ofw_ctx *o, const char *name, double v);

/* INITIALIZATION (init.F:280-1272) for a case whose interior Depth (and,
 * optionally, interior Eta/U/V) have been written into the fields first. */
int  ofw_init(ofw_ctx *o);
/* JON_2D random phases phi1(kf,ktheta) (kf fastest, nfreq*ntheta values);
 * the reference draws them from the compiler's rand(0), so they are
 * injected.  Call before ofw_init. */
void ofw_set_phases(ofw_ctx *o, const double *phi1);
/* JON_2D results of ofw_init: omega_k (nfreq), the band Cm/Sm (band-major:
 * i fastest, then j, then k; size (ihi-ilo+1)*(jhi-jlo+1)*nfreq). */
const double *ofw_jon_omega(ofw_ctx *o);
const double *ofw_jon_cm(ofw_ctx *o);
const double *ofw_jon_sm(ofw_ctx *o);
/* JON_2D spectrum tables of ofw_init: D_gen(kf,kt), rlamda(kf,kt)
 * (kf fastest) and beta_gen(kf). */
const double *ofw_jon_dgen(ofw_ctx *o);
const double *ofw_jon_rlamda(ofw_ctx *o);
const double *ofw_jon_betagen(ofw_ctx *o);

/* One step of main.F:284-535 (without OUTPUT).  Returns 0, or 1 when
 * CHECK_BLOWUP would stop the run. */
int  ofw_step(ofw_ctx *o);

/* Individual subroutines (the reference's argument-less units). */
void ofw_exchange(ofw_ctx *o);                 /* bc.F:426 */
void ofw_estimate_dt(ofw_ctx *o);              /* misc.F:216 */
void ofw_cal_dispersion(ofw_ctx *o);           /* dispersion.F:62 */
void ofw_fluxes(ofw_ctx *o);                   /* fluxes.F:52 */
void ofw_source_terms(ofw_ctx *o);             /* sources.F:56 */
void ofw_estimate_huv(ofw_ctx *o, int istage); /* etauv_solver.F:53 */
void ofw_update_mask(ofw_ctx *o);              /* masks.F:51 */
void ofw_wave_breaking(ofw_ctx *o);            /* breaker.F:60 */
void ofw_sponge_damping(ofw_ctx *o);           /* sponge.F:52 */
void ofw_begin_step(ofw_ctx *o);               /* main.F:295-331 */
void ofw_stage(ofw_ctx *o, int istage);        /* main.F:382-485 */
int  ofw_check_blowup(ofw_ctx *o);             /* misc.F:394 */
void ofw_max_min_property(ofw_ctx *o);         /* misc.F:307 (Hmax, Hmin, Umax, MFmax) */
void ofw_mixing_stuff(ofw_ctx *o);             /* mixing.F:53 (CALCULATE_MEAN, time means and wave heights) */
int  ofw_end_step(ofw_ctx *o);                 /* main.F:496-517: MIXING_STUFF, MAX_MIN_PROPERTY, CHECK_BLOWUP */

/* Bytes of the arithmetic type: 8 for the FP64 build (the checker), 4 for
 * the single-precision build that only the CPU baseline times.  Field
 * arrays (ofw_field) hold that type; masks stay int32. */
int ofw_real_bytes(void);

/* OpenMP threads used by the parallel-safe loops (0 = library default). */
void ofw_set_threads(int n);
int  ofw_get_threads(void);

#ifdef __cplusplus
}
#endif
#endif
