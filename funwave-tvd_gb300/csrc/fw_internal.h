// fw_internal.h -- device state and launch interface of the GB300 solver.
//
// Device layout: every 2-D field (cells, x-faces, y-faces) is stored
// x-fastest with one common pitch (elements) >= Mloc+1, rounded up to 32
// elements, and Nloc+1 rows; index (i, j) -> i + j*pitch with 0-based i, j
// (Fortran I = i+1).  Bulk fields are T (double in FP64 mode, float in mixed
// mode); masks are uint8; the tridiagonal u/v recovery works in double.
#pragma once

#include <cstddef>
#include <cstdint>

#include <cuda.h>

#include "funwave_gpu.h"

namespace fw {

constexpr int NG = 3;  // Nghost (mod_global.F:129)

// Scalars every kernel needs, passed by value.
struct Grid {
    int Mloc, Nloc, pitch;
    int ib, ie, jb, je;      // 0-based interior bounds, inclusive
    int Mglob, Nglob;
    int periodic, dispersion, visc_breaking, show_breaking;
    int direct_sponge, friction_sponge, eta_limiter, wavemaker;
    int ilo, ihi, jlo, jhi;  // 0-based wavemaker band (empty when ilo > ihi)
    int nfreq;
    int has_g2;              // Gamma2 > 0 (the dispersive ETAx/ETAy exchange)
    int track_hmin, track_umax, track_mfmax, stats;  // statistics switches
    int track_roller;        // BREAKING's roller flux and undertow (ROLLER / UNDERTOW output)
    int track_rad;           // CALCULATE_MEAN's radiation-stress, momentum-flux, dissipation sums
    int brk_passes;          // fixed-point passes of the breaking sweep before the level-ordered one
    double steady_time, t_intv_mean;
    double DX, DY;
    double gamma1, gamma2, gamma3, b1, b2, Beta_1, Beta_2;
    double cbrk1, cbrk2, wavemaker_cbrk, nu_bkg, T_brk;
    double swe_eta_dep, froude_cap, min_depth_frc, cfl, dt_fixed;
    int fixed_dt;
    double trough, crest;
    double xc_wk, yc_wk, ywidth_wk, width_wk;
    double D_gen, beta_gen, rlamda, tperiod, time_ramp, freq_peak;
    // constants of the mixed path: tridiagonal coefficient factors per
    // direction (b1/2/h^2, b2/h^2, (-b1-2*b2)/h^2) and 1/DX, 1/DY
    double cA[2], cB[2], cC[2];
    // FP64 path: b1/2/h/h, b2/h/h, -b1/h/h, 2*b2/h/h per direction, in the
    // reference's evaluation order
    double tK1[2], tK2[2], tK3[2], tK4[2];
    double rdx, rdy;
    // float copies of the constants for the mixed path (no FP64 work per
    // thread there): f_<name> = (float)<name>; f_hdx = 0.5/DX, f_rdx2 =
    // 1/DX^2, f_rdxy4 = 0.25/(DX*DY), f_cx = 0.5/DX^2, f_hb1 = -0.5*b1
    float f_DX, f_DY, f_rdx, f_rdy, f_hdx, f_hdy, f_rdx2, f_rdy2, f_rdxy4, f_cx, f_cy;
    float f_min_depth_frc, f_gamma1, f_gamma2, f_gamma3, f_Beta_1, f_Beta_2, f_b1, f_b2, f_hb1;
    float f_cbrk1, f_cbrk2, f_wavemaker_cbrk, f_nu_bkg, f_T_brk, f_froude_cap, f_swe_eta_dep;
    float f_xc_wk, f_yc_wk, f_ywidth_wk, f_width_wk, f_D_gen, f_beta_gen, f_rlamda, f_trough, f_crest;
};

// float device scalars of the current step (mixed path)
enum : int { FS_DT = 0, FS_RDT = 1, FS_WKAA = 2, FS_WKPH = 3, FS_TSUM = 4, FS_NSLOT = 8 };

// device scalar slots (double array)
// S_TSUM: T_sum of MIXING_STUFF; S_TSUMU: the T_sum this step's means use;
// S_MFLAG: 0 no statistics this step, 1 accumulate, 2 end of an interval;
// S_NMEAN: intervals ended so far (the reference's ICOUNT_MEAN, io.F:4641)
enum : int {
    S_TIME = 0, S_DT = 1, S_DTMIN = 2, S_ETAMAX = 3, S_TSUM = 4, S_TSUMU = 5, S_MFLAG = 6, S_NMEAN = 7, S_NSLOT = 8
};

template <typename T>
struct Fields {
    T *Eta, *U, *V, *Ubar, *Vbar, *HU, *HV, *H;
    T *Eta0, *Ubar0, *Vbar0, *U0, *V0;
    T *Depth, *Depthx, *Depthy, *Cd, *SPONGE, *CD4;
    T *P, *Q, *Fx, *Fy, *Gx, *Gy;
    T *A, *B, *C, *E;                 // mixed: exchanged Uxx+Vxy, DUxx+DVxy, Uxy+Vyy, DUxy+DVyy
    T *Uxx, *Vxy, *Uxy, *Vyy, *DUxx, *DVxy, *DUxy, *DVyy;  // FP64: the exchanged terms themselves
    T *U4, *V4, *U1p, *V1p, *Udisp, *Vdisp;  // Udisp = U1pp+U2+U3
    T *ETAx, *ETAy, *ETAT;
    T *AGE, *AGEn, *nu;               // AGE ping-pong (old / new)
    T *SourceX, *SourceY, *WM;        // materialised only by the unit entry points
    T *Hmax;
    // statistics (null unless switched on): MAX_MIN_PROPERTY and CALCULATE_MEAN
    T *Hmin, *Umax, *MFmax;
    T *ETAmean, *Umean, *Vmean, *ETAsum, *Usum, *Vsum, *ETA2sum, *ETA2mean, *SigWH, *Emax, *Emin, *HavgSum,
        *HrmsSum, *WHave, *WHrms, *NZU;
    T *kETAsum, *kUsum, *kVsum, *kETA2sum;  // Kahan compensations of the mixed path
    T *ROLLER, *UNDERTOW_U, *UNDERTOW_V;    // breaker.F:316-339 (null unless tracked)
    T *rad;  // radiation-stress planes (fw::RadPlane), consecutive planes of the field plane size; null if off
    uint8_t *MASK, *MASKn, *MASK9, *MASK_STRUC;
    T *rhs_x, *rhs_y;                 // tmp4 of GET_Eta_U_V_HU_HV
    double *ty, *tp, *tq, *tc;        // line-solver scratch
    // Depth as the caller gave it, in double: the FP64 build's Depth itself;
    // in the mixed build a copy that UPDATE_MASK's total-depth tests read
    double *DepthD;
    double *sw_p[2], *sw_q[2], *sw_c[2];  // factorisation sweep scratch per direction (mixed)
    double *red;                      // reduced systems
    // mixed path: constant factorisation of the tridiagonal matrices, per
    // direction d, rounded to float: per row d-scale (1/tmp2, times r on
    // chunk interiors), lower*r, c', p, q and the normalised coefficients a,
    // c as float pairs (hi + lo) for the compensated residual; per reduced
    // row lo, 1/den, c'; per chunk c_s, a_e; per line (periodic) the second
    // solution, c_end, a_beg and the Sherman-Morrison denominator
    float *fac_it[2], *fac_A[2], *fac_lr[2], *fac_cp[2], *fac_p[2], *fac_q[2];
    float *fac_ah[2], *fac_al[2], *fac_ch[2], *fac_cl[2];
    float *fac_red[2];
    int *m9_dirty;                    // MASK9 changed since the last factorisation
    T *Cm, *Sm;                       // JON_2D band tables (in the field precision)
    double *omega, *wmcs;             // JON_2D frequencies and cos/sin(omega t)
    double *dsc;                      // device scalars (S_*)
    float *fsc;                       // float device scalars (FS_*)
    float *wmcsf;                     // float copy of wmcs
    int *cand, *ncand;                // breaking candidates
    unsigned long long *dtmin_bits;
    unsigned long long *etamax_bits;
};

// the planes behind Fields::rad: the per-step inputs that ESTIMATE_HUV and
// SourceTerms leave at the last stage (etauv_solver.F:94-101, 247;
// sources.F:428-456), twelve time sums, their twelve means and the ten
// gradient fields of CALCULATE_MEAN (mixing.F:156-219); the mixed path adds
// the sums' Kahan compensations.  Sums and means share one order:
// U_davg, V_davg, P_center, Q_center, UU, UV, VV, WW, FRCX, FRCY,
// BreakDissX, BreakDissY
enum RadPlane {
    RP_PC, RP_QC, RP_UD, RP_VD, RP_WS, RP_BX, RP_BY,
    RP_SUM = 7,
    RP_MEAN = RP_SUM + 12,
    RP_DER = RP_MEAN + 12,  // DxSxx, DySxy, DySyy, DxSxy, PgrdX, PgrdY, DxUUH, DyUVH, DyVVH, DxUVH
    RP_KAHAN = RP_DER + 10,
    RP_N64 = RP_KAHAN,
    RP_N32 = RP_KAHAN + 12
};

// line-solver partition of one direction
struct LinePart {
    int L;       // line length (interior rows)
    int nlines;  // number of lines
    int m;       // rows per chunk (the last chunk takes the remainder)
    int P;       // chunks per line
    long long red0;  // offset (doubles) of this direction's rows in the factorisation scratch
    int lgm;         // log2(m) when m is a power of two, else -1
};

// launchers (fw_kernels.cu), all asynchronous on the context stream
template <typename T> void launch_begin_step(fw_ctx *c);
template <typename T> void launch_exchange(fw_ctx *c, bool with_sponge);
template <typename T> void launch_estimate_dt(fw_ctx *c);
template <typename T> void launch_dispersion(fw_ctx *c);
template <typename T> void launch_fluxes(fw_ctx *c);
template <typename T> void launch_sources_debug(fw_ctx *c);
template <typename T> void launch_estimate_huv(fw_ctx *c, int istage);
template <typename T> void launch_update_mask(fw_ctx *c);
template <typename T> void launch_breaking(fw_ctx *c);
template <typename T> void launch_sponge(fw_ctx *c);
template <typename T> void launch_end_step(fw_ctx *c);
template <typename T> void launch_stage(fw_ctx *c, int istage);
void gather_points(fw_ctx *c, const void *field, int type, const int *d_off, int n, double *d_out);
template <typename T>
void launch_cm_sm(fw_ctx *c, int bw, int bh, int i0, int j0, const double *tab, T *Cm, T *Sm);
template <typename T> int launch_by_name(fw_ctx *c, const char *name);
template <typename T> bool flux_tma_attrs();  // shared-memory sizes of the TMA-staged flux kernels
// staging buffer <-> field (double <-> float fields, int32 <-> uint8 masks)
void convert_in(fw_ctx *c, const void *staging, int is_mask, void *field, int w, int h);
void convert_out(fw_ctx *c, const void *field, int is_mask, void *staging, int w, int h);
void convert_in_f32(fw_ctx *c, const float *staging, double *field, int w, int h);
void convert_out_f32(fw_ctx *c, const double *field, float *staging, int w, int h);

}  // namespace fw

#include <cuda_runtime.h>

// Host context behind the opaque C handle.
namespace fw {
// tensor maps of the flux kernels' TMA-staged tiles: U V HU HV Eta U4 V4 and
// MASK, for one direction and tile height (the box shape is part of a map)
// and one of the two MASK buffers
struct FluxMaps {
    CUtensorMap m[8];
    // polls of the wait for the staged tile before the block gives up and
    // writes NaN fluxes (which the step reports); 0 = the default limit.
    // Set through fw_set_scalar("WAIT_LIMIT").
    unsigned wait_limit;
};
constexpr int FLUX_FY_N = 3;  // tile heights 8, 16, 32
// kernels whose block shape fw_autotune chooses (per-cell kernels, so any
// shape gives the same results); the tuning vector holds (bx, by) for each,
// then the tile heights of the x and y flux kernels (FW_TUNE_LEN ints)
enum TuneKernel { TK_DISP_A = 0, TK_DISP_B, TK_UPDATE, TK_PMB, TK_MASKMUL, TK_N };
constexpr int TUNE_FLUX = 2 * TK_N;      // flux tile heights (x, y)
constexpr int TUNE_FLUX_TMA = 2 * TK_N + 2;  // flux staging by TMA (x, y): 0 loads, 1 TMA
}  // namespace fw

struct fw_ctx {
    fw_params p;
    int tune[FW_TUNE_LEN] = {32, 8, 32, 8, 32, 8, 32, 8, 32, 8, 8, 32, 0, 0};  // see fw::TuneKernel
    // the flux kernels' tensor maps: [direction][tile height 8/16/32][MASK buffer]
    fw::FluxMaps fmaps[2][fw::FLUX_FY_N][2];
    const void *fmask_base[2] = {nullptr, nullptr};  // the two MASK buffers the maps were made for
    int fmaps_ok = 0;
    dim3 blk(int k) const { return dim3((unsigned)tune[2 * k], (unsigned)tune[2 * k + 1]); }
    fw::Grid g;
    cudaStream_t stream = nullptr;
    fw::Fields<double> fd{};
    fw::Fields<float> ff{};
    fw::LinePart px{}, py{};
    void *arena = nullptr;       // one device allocation holds every field
    void *staging = nullptr;     // one host-layout plane for field transfers
    size_t arena_bytes = 0;
    int ncand_cap = 0;
    long long launches = 0;
    int initialized = 0;
    int sticky_error = 0;        // first CUDA error seen by a launcher
    double EtaBlowVal = 0.0;
    cudaGraphExec_t graph = nullptr;
    int graph_ready = 0;
    int factored = 0;            // mixed path solves with the constant factorisation
    long long graph_state = 0;   // host buffer state the graph was captured with
    // one-step graphs, one per ping-pong orientation (fw_step(ctx, 1, ...)
    // as a time loop with the reference's shape calls it)
    cudaGraphExec_t graph1[2] = {nullptr, nullptr};
    long long graph1_state[2] = {0, 0};
    // the MASK, MASKn, AGE, AGEn pointers after each graph's step: a replay
    // does not run the host-side swaps that capturing the step did
    void *graph1_post[2][4] = {};
    int graph1_ok[2] = {0, 0};
    int graph1_next = 0;
    void invalidate_graphs() { graph_ready = graph1_ok[0] = graph1_ok[1] = 0; }
    // asynchronous output (fw_output_begin / fw_output_wait): host-layout
    // snapshots in out_buf, copied to the caller's buffers on out_stream
    void *out_buf = nullptr;
    size_t out_cap = 0;
    cudaStream_t out_stream = nullptr;
    cudaEvent_t out_ready = nullptr, out_done = nullptr;
    int out_pending = 0;
    // batched uploads (fw_set_fields): host-layout planes in in_buf, one
    // event per plane
    void *in_buf = nullptr;
    size_t in_cap = 0;
    cudaEvent_t in_ev[16] = {};
    template <typename T> fw::Fields<T> &F();
};
namespace fw {
// stepping pieces for other translation units (fw_api.cu)
int enqueue_one_step(fw_ctx *c);          // one whole step on c->stream, no graph
int reset_step_max(fw_ctx *c);            // CHECK_BLOWUP's maximum, before a run of steps
int step_status(fw_ctx *c, int *status);  // waits for c->stream; FW_OK or the run's status
long long buffer_state(fw_ctx *c);        // the host pointer state a captured step bakes in
}  // namespace fw

template <> inline fw::Fields<double> &fw_ctx::F<double>() { return fd; }
template <> inline fw::Fields<float> &fw_ctx::F<float>() { return ff; }
