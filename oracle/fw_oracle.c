/*
 * fw_oracle.c -- FP64 CPU restatement of the FUNWAVE-TVD SSP-RK3 stage.
 *
 * TEST INFRASTRUCTURE ONLY (checker and timed CPU baseline); see fw_oracle.h.
 * Parity unpinned against the Fortran itself (no Fortran compiler, no golden
 * vectors in the reference); pinned by the invariants and known-answer cases
 * in tests/.
 *
 * Each function follows one reference subroutine statement by statement,
 * keeping its loop ranges, its in-place update order and its operand order
 * (compile with -ffp-contract=off).  Where the reference reads memory that
 * it never initialises, this restatement defines the value and says so:
 *   - MASK9 outside Ibeg-1..Iend+1 x Jbeg-1..Jend+1 (masks.F:175-193 copies a
 *     freshly ALLOCATEd temporary whose outer ring is never written) is 0,
 *     i.e. zero-filled memory; MASK9 at initialisation is 0 outside the
 *     interior (init.F:1153-1159) and 0 everywhere before that point.
 *   - BREAKING's local DXg/DYg (breaker.F:98-100,123-124) are DX/DY.
 *   - DT before the first ESTIMATE_DT is 0 (module variable).
 * Default-REAL literals of the FP64 build are widened from float with
 * (ofr)(float)x (mod_param.F:71 pi, wavemaker.F:2378-2399), and nu_vis is
 * a float array (sources.F:69).
 */
#include "fw_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* The arithmetic type.  The default build is the FP64 restatement.  With
 * OFW_FP32 (and -fsingle-precision-constant) the same source is a single-
 * precision build, as the reference's default REAL(SP) = 4-byte build is
 * (mod_param.F:58-68): every real and literal is a float and the math
 * functions are their float forms.  It serves only the CPU baseline's
 * timing; the checker is the FP64 build. */
#ifdef OFW_FP32
typedef float ofr;
#define sqrt sqrtf
#define fabs fabsf
#define exp expf
#define sin sinf
#define cos cosf
#define tanh tanhf
#define atan2 atan2f
#define pow powf
#define copysign copysignf
#define asin asinf
#else
typedef double ofr;
#endif

int ofw_real_bytes(void) { return (int)sizeof(ofr); }

#define GRAV 9.81
#define SMALL 0.000001
#define LARGE 999999.0
#define ZERO 0.0
#define NGHOST 3

/* pi is a default-REAL literal assigned to REAL(SP) (mod_param.F:71). */
static const ofr PI_SP = (ofr)(float)3.141592653;

struct ofw_ctx {
    ofw_params p;
    int Mloc, Nloc, Mloc1, Nloc1, Ibeg, Iend, Jbeg, Jend, Iend1, Jend1;
    ofr TIME, DT, T_brk, EtaBlowVal;
    ofr a1, a2, b1, b2, Beta_1, Beta_2;
    ofr D_gen, beta_gen, rlamda, Width_WK;
    int ilo, ihi, jlo, jhi;
    ofr *xmk_wk, *ymk_wk;
    double *omgn_ir, *Cm, *Sm; /* JON_2D band storage */
    double *phi1, *jon_dgen, *jon_rlamda, *jon_betagen;
    /* cell arrays */
    ofr *Depth, *H, *Eta, *Eta0, *U, *V, *U0, *V0, *Ubar, *Vbar, *Ubar0,
        *Vbar0, *HU, *HV, *Cd, *SPONGE, *CD_4_SPONGE, *ETAT, *ETAx, *ETAy, *Ux,
        *Vx, *Uy, *Vy, *DUx, *DVx, *DUy, *DVy, *Uxx, *Uxy, *Vxy, *Vyy, *DUxx,
        *DUxy, *DVxy, *DVyy, *Ut, *Vt, *Utx, *Vty, *Utxx, *Utxy, *Vtxy, *Vtyy,
        *DUtx, *DVty, *DUtxx, *DUtxy, *DVtxy, *DVtyy, *U4, *V4, *U1p, *V1p,
        *U1pp, *V1pp, *U2, *V2, *U3, *V3, *SourceX, *SourceY, *WaveMaker_Mass,
        *AGE, *nu_break, *HeightMax, *ROLLER_FLUX, *UNDERTOW_U, *UNDERTOW_V;
    /* statistics: MAX_MIN_PROPERTY and CALCULATE_MEAN */
    ofr T_sum;
    ofr *HeightMin, *VelocityMax, *MomentumFluxMax, *ETAmean, *Umean, *Vmean, *ETAsum, *Usum, *Vsum,
        *ETA2sum, *ETA2mean, *SigWaveHeight, *Emax, *Emin, *HavgSum, *HrmsSum, *WaveHeightAve, *WaveHeightRMS;
    int *Num_Zero_Up;
    /* radiation stress, momentum flux and breaking dissipation of
     * CALCULATE_MEAN (mixing.F:156-200), with their per-stage inputs from
     * ESTIMATE_HUV (etauv_solver.F:94-101, 247) and SourceTerms
     * (sources.F:428-456) */
    ofr *P_center, *Q_center, *U_davg, *V_davg, *Wsurf, *BreakSourceX, *BreakSourceY;
    ofr *U_davg_sum, *V_davg_sum, *P_sum, *Q_sum, *UUsum, *UVsum, *VVsum, *WWsum, *FRCXsum, *FRCYsum,
        *BreakDissX_sum, *BreakDissY_sum;
    ofr *U_davg_mean, *V_davg_mean, *P_mean, *Q_mean, *UUmean, *UVmean, *VVmean, *WWmean, *FRCXmean,
        *FRCYmean, *BreakDissX, *BreakDissY;
    ofr *DxSxx, *DySxy, *DySyy, *DxSxy, *PgrdX, *PgrdY, *DxUUH, *DyUVH, *DyVVH, *DxUVH;
    int *MASK, *MASK9, *MASK_STRUC;
    /* x-face arrays */
    ofr *Depthx, *P, *Fx, *Gx, *UxL, *UxR, *VxL, *VxR, *HUxL, *HUxR, *HVxL,
        *HVxR, *EtaRxL, *EtaRxR, *HxL, *HxR, *U4xL, *U4xR, *V4xL, *V4xR, *PL,
        *PR, *FxL, *FxR, *GxL, *GxR, *SxL, *SxR;
    /* y-face arrays */
    ofr *Depthy, *Q, *Fy, *Gy, *UyL, *UyR, *VyL, *VyR, *HUyL, *HUyR, *HVyL,
        *HVyR, *EtaRyL, *EtaRyR, *HyL, *HyR, *U4yL, *U4yR, *V4yL, *V4yR, *QL,
        *QR, *FyL, *FyR, *GyL, *GyR, *SyL, *SyR;
};

/* 1-based Fortran indexing. */
#define C2(a, I, J) (a)[(size_t)((I)-1) + (size_t)((J)-1) * (size_t)o->Mloc]
#define X2(a, I, J) (a)[(size_t)((I)-1) + (size_t)((J)-1) * (size_t)o->Mloc1]
#define Y2(a, I, J) C2(a, I, J)

static int g_threads = 0;
void ofw_set_threads(int n) { g_threads = n; }
int ofw_get_threads(void) {
#ifdef _OPENMP
    return g_threads > 0 ? g_threads : omp_get_max_threads();
#else
    return 1;
#endif
}
#ifdef _OPENMP
#define OMP_FOR _Pragma("omp parallel for num_threads(ofw_get_threads()) schedule(static)")
#else
#define OMP_FOR
#endif

static inline ofr dmax(ofr a, ofr b) { return a > b ? a : b; }
static inline ofr dmin(ofr a, ofr b) { return a < b ? a : b; }
/* Fortran MAX(a,b,c) / MIN(a,b,c) */
static inline ofr max3(ofr a, ofr b, ofr c) { return dmax(dmax(a, b), c); }
static inline ofr min3(ofr a, ofr b, ofr c) { return dmin(dmin(a, b), c); }

/* ------------------------------------------------------------------------ */
/* construction / field table                                               */
/* ------------------------------------------------------------------------ */

typedef struct { const char *name; size_t off; int kind; int is_int; } field_desc;
#define FD(n, k) {#n, offsetof(struct ofw_ctx, n), k, 0}
#define FI(n, k) {#n, offsetof(struct ofw_ctx, n), k, 1}
#include <stddef.h>
static const field_desc FIELDS[] = {
    FD(Depth, 0), FD(H, 0), FD(Eta, 0), FD(Eta0, 0), FD(U, 0), FD(V, 0),
    FD(U0, 0), FD(V0, 0), FD(Ubar, 0), FD(Vbar, 0), FD(Ubar0, 0), FD(Vbar0, 0),
    FD(HU, 0), FD(HV, 0), FD(Cd, 0), FD(SPONGE, 0), FD(CD_4_SPONGE, 0),
    FD(ETAT, 0), FD(ETAx, 0), FD(ETAy, 0), FD(Ux, 0), FD(Vx, 0), FD(Uy, 0),
    FD(Vy, 0), FD(DUx, 0), FD(DVx, 0), FD(DUy, 0), FD(DVy, 0), FD(Uxx, 0),
    FD(Uxy, 0), FD(Vxy, 0), FD(Vyy, 0), FD(DUxx, 0), FD(DUxy, 0), FD(DVxy, 0),
    FD(DVyy, 0), FD(Ut, 0), FD(Vt, 0), FD(Utx, 0), FD(Vty, 0), FD(Utxx, 0),
    FD(Utxy, 0), FD(Vtxy, 0), FD(Vtyy, 0), FD(DUtx, 0), FD(DVty, 0),
    FD(DUtxx, 0), FD(DUtxy, 0), FD(DVtxy, 0), FD(DVtyy, 0), FD(U4, 0),
    FD(V4, 0), FD(U1p, 0), FD(V1p, 0), FD(U1pp, 0), FD(V1pp, 0), FD(U2, 0),
    FD(V2, 0), FD(U3, 0), FD(V3, 0), FD(SourceX, 0), FD(SourceY, 0),
    FD(WaveMaker_Mass, 0), FD(AGE, 0), FD(nu_break, 0), FD(HeightMax, 0),
    FD(ROLLER_FLUX, 0), FD(UNDERTOW_U, 0), FD(UNDERTOW_V, 0),
    FD(HeightMin, 0), FD(VelocityMax, 0), FD(MomentumFluxMax, 0), FD(ETAmean, 0), FD(Umean, 0),
    FD(Vmean, 0), FD(ETAsum, 0), FD(Usum, 0), FD(Vsum, 0), FD(ETA2sum, 0), FD(ETA2mean, 0),
    FD(SigWaveHeight, 0), FD(Emax, 0), FD(Emin, 0), FD(HavgSum, 0), FD(HrmsSum, 0),
    FD(WaveHeightAve, 0), FD(WaveHeightRMS, 0), FI(Num_Zero_Up, 0),
    FD(P_center, 0), FD(Q_center, 0), FD(U_davg, 0), FD(V_davg, 0), FD(Wsurf, 0), FD(BreakSourceX, 0),
    FD(BreakSourceY, 0), FD(U_davg_sum, 0), FD(V_davg_sum, 0), FD(P_sum, 0), FD(Q_sum, 0), FD(UUsum, 0),
    FD(UVsum, 0), FD(VVsum, 0), FD(WWsum, 0), FD(FRCXsum, 0), FD(FRCYsum, 0), FD(BreakDissX_sum, 0),
    FD(BreakDissY_sum, 0), FD(U_davg_mean, 0), FD(V_davg_mean, 0), FD(P_mean, 0), FD(Q_mean, 0), FD(UUmean, 0),
    FD(UVmean, 0), FD(VVmean, 0), FD(WWmean, 0), FD(FRCXmean, 0), FD(FRCYmean, 0), FD(BreakDissX, 0),
    FD(BreakDissY, 0), FD(DxSxx, 0), FD(DySxy, 0), FD(DySyy, 0), FD(DxSxy, 0), FD(PgrdX, 0), FD(PgrdY, 0),
    FD(DxUUH, 0), FD(DyUVH, 0), FD(DyVVH, 0), FD(DxUVH, 0),
    FI(MASK, 0), FI(MASK9, 0), FI(MASK_STRUC, 0),
    FD(Depthx, 1), FD(P, 1), FD(Fx, 1), FD(Gx, 1), FD(UxL, 1), FD(UxR, 1),
    FD(VxL, 1), FD(VxR, 1), FD(HUxL, 1), FD(HUxR, 1), FD(HVxL, 1), FD(HVxR, 1),
    FD(EtaRxL, 1), FD(EtaRxR, 1), FD(HxL, 1), FD(HxR, 1), FD(U4xL, 1),
    FD(U4xR, 1), FD(V4xL, 1), FD(V4xR, 1), FD(PL, 1), FD(PR, 1), FD(FxL, 1),
    FD(FxR, 1), FD(GxL, 1), FD(GxR, 1), FD(SxL, 1), FD(SxR, 1),
    FD(Depthy, 2), FD(Q, 2), FD(Fy, 2), FD(Gy, 2), FD(UyL, 2), FD(UyR, 2),
    FD(VyL, 2), FD(VyR, 2), FD(HUyL, 2), FD(HUyR, 2), FD(HVyL, 2), FD(HVyR, 2),
    FD(EtaRyL, 2), FD(EtaRyR, 2), FD(HyL, 2), FD(HyR, 2), FD(U4yL, 2),
    FD(U4yR, 2), FD(V4yL, 2), FD(V4yR, 2), FD(QL, 2), FD(QR, 2), FD(FyL, 2),
    FD(FyR, 2), FD(GyL, 2), FD(GyR, 2), FD(SyL, 2), FD(SyR, 2),
};
#define NFIELDS (sizeof(FIELDS) / sizeof(FIELDS[0]))

ofw_ctx *ofw_create(const ofw_params *p) {
    ofw_ctx *o = (ofw_ctx *)calloc(1, sizeof(ofw_ctx));
    if (!o) return NULL;
    o->p = *p;
    /* INDEX, serial branch (misc.F:160-176) */
    o->Mloc = p->Mglob + 2 * NGHOST;
    o->Nloc = p->Nglob + 2 * NGHOST;
    o->Mloc1 = o->Mloc + 1;
    o->Nloc1 = o->Nloc + 1;
    o->Ibeg = NGHOST + 1;
    o->Iend = o->Mloc - NGHOST;
    o->Iend1 = o->Mloc1 - NGHOST;
    o->Jbeg = NGHOST + 1;
    o->Jend = o->Nloc - NGHOST;
    o->Jend1 = o->Nloc1 - NGHOST;
    size_t nc = (size_t)o->Mloc * o->Nloc;
    size_t nx = (size_t)o->Mloc1 * o->Nloc;
    size_t ny = (size_t)o->Mloc * o->Nloc1;
    for (size_t k = 0; k < NFIELDS; k++) {
        size_t n = FIELDS[k].kind == 0 ? nc : FIELDS[k].kind == 1 ? nx : ny;
        void *buf = calloc(n, FIELDS[k].is_int ? sizeof(int) : sizeof(ofr));
        if (!buf) { ofw_destroy(o); return NULL; }
        *(void **)((char *)o + FIELDS[k].off) = buf;
    }
    o->xmk_wk = (ofr *)calloc((size_t)o->Mloc, sizeof(ofr));
    o->ymk_wk = (ofr *)calloc((size_t)o->Nloc, sizeof(ofr));
    /* ALLOCATE_VARIABLES / INITIALIZATION defaults (init.F:445-560,624,214) */
    for (size_t k = 0; k < nc; k++) {
        o->Depth[k] = 10.0;
        o->MASK[k] = 1;
        o->MASK_STRUC[k] = 1;
        o->SPONGE[k] = 1.0;
        o->nu_break[k] = p->nu_bkg;
    }
    return o;
}

void ofw_destroy(ofw_ctx *o) {
    if (!o) return;
    for (size_t k = 0; k < NFIELDS; k++) free(*(void **)((char *)o + FIELDS[k].off));
    free(o->xmk_wk);
    free(o->ymk_wk);
    free(o->omgn_ir);
    free(o->Cm);
    free(o->Sm);
    free(o->phi1);
    free(o->jon_dgen);
    free(o->jon_rlamda);
    free(o->jon_betagen);
    free(o);
}

void *ofw_field(ofw_ctx *o, const char *name, int *kind, int *is_int) {
    for (size_t k = 0; k < NFIELDS; k++)
        if (strcmp(FIELDS[k].name, name) == 0) {
            if (kind) *kind = FIELDS[k].kind;
            if (is_int) *is_int = FIELDS[k].is_int;
            return *(void **)((char *)o + FIELDS[k].off);
        }
    return NULL;
}

double ofw_get_scalar(ofw_ctx *o, const char *n) {
    if (!strcmp(n, "TIME")) return o->TIME;
    if (!strcmp(n, "DT")) return o->DT;
    if (!strcmp(n, "T_brk")) return o->T_brk;
    if (!strcmp(n, "EtaBlowVal")) return o->EtaBlowVal;
    if (!strcmp(n, "D_gen")) return o->D_gen;
    if (!strcmp(n, "beta_gen")) return o->beta_gen;
    if (!strcmp(n, "rlamda")) return o->rlamda;
    if (!strcmp(n, "Width_WK")) return o->Width_WK;
    if (!strcmp(n, "ilo")) return o->ilo;
    if (!strcmp(n, "ihi")) return o->ihi;
    if (!strcmp(n, "jlo")) return o->jlo;
    if (!strcmp(n, "jhi")) return o->jhi;
    if (!strcmp(n, "T_sum")) return o->T_sum;
    return NAN;
}

void ofw_set_scalar(ofw_ctx *o, const char *n, double v) {
    if (!strcmp(n, "TIME")) o->TIME = v;
    else if (!strcmp(n, "DT")) o->DT = v;
    else if (!strcmp(n, "T_brk")) o->T_brk = v;
    else if (!strcmp(n, "EtaBlowVal")) o->EtaBlowVal = v;
    else if (!strcmp(n, "Width_WK")) o->Width_WK = v;
}

/* ------------------------------------------------------------------------ */
/* ghost-cell fill: PHI_COLL serial branches (bc.F:631-1272)                */
/* ------------------------------------------------------------------------ */

/* PHI_COLL(Mloc,Nloc,Ibeg,Iend,Jbeg,Jend,Nghost,PHI,VTYPE,PERIODIC) for a
 * cell array (bc.F:631-1272; periodic serial copy :735-740, VTYPE 1
 * :753-844, VTYPE 2 :847-937, VTYPE 3 :939-1029). */
static void phi_coll(ofw_ctx *o, ofr *PHI, int vtype) {
    const int M = o->Mloc, Ib = o->Ibeg, Ie = o->Iend, Jb = o->Jbeg, Je = o->Jend;
    const int per = o->p.periodic;
    if (per) {
        for (int I = 1; I <= M; I++)
            for (int K = 1; K <= NGHOST; K++) {
                C2(PHI, I, K) = C2(PHI, I, Je - NGHOST + K);
                C2(PHI, I, Je + K) = C2(PHI, I, NGHOST + K);
            }
    }
    const ofr sx = (vtype == 2) ? -1.0 : 1.0; /* u: x-antisymmetric */
    const ofr sy = (vtype == 3) ? -1.0 : 1.0; /* v: y-antisymmetric */
    for (int J = Jb; J <= Je; J++)
        for (int K = 1; K <= NGHOST; K++) {
            ofr w = C2(PHI, Ib + NGHOST - K, J);
            C2(PHI, K, J) = (vtype == 2) ? -w : w;
        }
    for (int J = Jb; J <= Je; J++)
        for (int K = 1; K <= NGHOST; K++) {
            ofr e = C2(PHI, Ie - K + 1, J);
            C2(PHI, Ie + K, J) = (vtype == 2) ? -e : e;
        }
    (void)sx;
    if (!per) {
        for (int I = 1; I <= M; I++)
            for (int K = 1; K <= NGHOST; K++) {
                ofr s = C2(PHI, I, Jb + NGHOST - K);
                C2(PHI, I, K) = (vtype == 3) ? -s : s;
            }
        for (int I = 1; I <= M; I++)
            for (int K = 1; K <= NGHOST; K++) {
                ofr n = C2(PHI, I, Je - K + 1);
                C2(PHI, I, Je + K) = (vtype == 3) ? -n : n;
            }
    }
    (void)sy;
}

/* MASK goes through a REAL copy (bc.F:449-451); the int copy is identical. */
static void phi_coll_int(ofw_ctx *o, int *PHI) {
    const int M = o->Mloc, Ib = o->Ibeg, Ie = o->Iend, Jb = o->Jbeg, Je = o->Jend;
    if (o->p.periodic) {
        for (int I = 1; I <= M; I++)
            for (int K = 1; K <= NGHOST; K++) {
                C2(PHI, I, K) = C2(PHI, I, Je - NGHOST + K);
                C2(PHI, I, Je + K) = C2(PHI, I, NGHOST + K);
            }
    }
    for (int J = Jb; J <= Je; J++)
        for (int K = 1; K <= NGHOST; K++) C2(PHI, K, J) = C2(PHI, Ib + NGHOST - K, J);
    for (int J = Jb; J <= Je; J++)
        for (int K = 1; K <= NGHOST; K++) C2(PHI, Ie + K, J) = C2(PHI, Ie - K + 1, J);
    if (!o->p.periodic) {
        for (int I = 1; I <= M; I++)
            for (int K = 1; K <= NGHOST; K++) C2(PHI, I, K) = C2(PHI, I, Jb + NGHOST - K);
        for (int I = 1; I <= M; I++)
            for (int K = 1; K <= NGHOST; K++) C2(PHI, I, Je + K) = C2(PHI, I, Je - K + 1);
    }
}

/* PHI_COLL_VARIABLE_LENGTH (bc.F:530-629), VTYPE 1: plain mirror on all four
 * sides, periodic ignored.  ld = leading dimension, (m,n) the extents,
 * ie/je the last interior index passed in (Iend1 for P, Jend1 for Q). */
static void phi_coll_var(ofw_ctx *o, ofr *PHI, int ld, int m, int ie, int je) {
    const int Ib = o->Ibeg, Jb = o->Jbeg;
#define V2(I, J) PHI[(size_t)((I)-1) + (size_t)((J)-1) * (size_t)ld]
    for (int J = Jb; J <= je; J++)
        for (int K = 1; K <= NGHOST; K++) V2(K, J) = V2(Ib + NGHOST - K, J);
    for (int J = Jb; J <= je; J++)
        for (int K = 1; K <= NGHOST; K++) V2(ie + K, J) = V2(ie - K + 1, J);
    for (int I = 1; I <= m; I++)
        for (int K = 1; K <= NGHOST; K++) V2(I, K) = V2(I, Jb + NGHOST - K);
    for (int I = 1; I <= m; I++)
        for (int K = 1; K <= NGHOST; K++) V2(I, je + K) = V2(I, je - K + 1);
#undef V2
}

/* EXCHANGE (bc.F:426-529), CARTESIAN.  Wsurf, P_center, Q_center, U_davg
 * and V_davg are output-only diagnostics and are not kept here. */
void ofw_exchange(ofw_ctx *o) {
    phi_coll(o, o->Eta, 1);
    /* for radiation stress (bc.F:438-443) */
    phi_coll(o, o->Wsurf, 1);
    phi_coll(o, o->P_center, 1);
    phi_coll(o, o->Q_center, 1);
    phi_coll(o, o->U_davg, 1);
    phi_coll(o, o->V_davg, 1);
    if (o->p.viscosity_breaking) phi_coll(o, o->AGE, 1);
    if (o->p.viscosity_breaking) phi_coll(o, o->nu_break, 1);
    if (o->p.viscosity_breaking) {
        phi_coll_var(o, o->P, o->Mloc1, o->Mloc1, o->Iend1, o->Jend);
        phi_coll_var(o, o->Q, o->Mloc, o->Mloc, o->Iend, o->Jend1);
    }
    phi_coll_int(o, o->MASK);
    phi_coll(o, o->U, 2);
    phi_coll(o, o->HU, 2);
    phi_coll(o, o->V, 3);
    phi_coll(o, o->HV, 3);
    const size_t nc = (size_t)o->Mloc * o->Nloc;
    OMP_FOR
    for (size_t k = 0; k < nc; k++) {
        ofr m = (ofr)o->MASK[k];
        o->U[k] = o->U[k] * m;
        o->V[k] = o->V[k] * m;
        o->HU[k] = o->HU[k] * m;
        o->HV[k] = o->HV[k] * m;
    }
}

/* ------------------------------------------------------------------------ */
/* ESTIMATE_DT (misc.F:216-296), CARTESIAN                                  */
/* ------------------------------------------------------------------------ */
void ofw_estimate_dt(ofw_ctx *o) {
    const ofr DX = o->p.DX, DY = o->p.DY, mdf = o->p.min_depth_frc;
    ofr TMP3 = LARGE;
    const int M = o->Mloc, N = o->Nloc;
#ifdef _OPENMP
#pragma omp parallel for num_threads(ofw_get_threads()) reduction(min : TMP3)
#endif
    for (int J = 1; J <= N; J++)
        for (int I = 1; I <= M; I++) {
            ofr c = sqrt(GRAV * dmax(C2(o->H, I, J), mdf));
            ofr TMP1 = fabs(C2(o->U, I, J)) + c;
            ofr TMP2 = (TMP1 < SMALL) ? DX / SMALL : DX / TMP1;
            if (TMP2 < TMP3) TMP3 = TMP2;
            TMP1 = fabs(C2(o->V, I, J)) + c;
            TMP2 = (TMP1 < SMALL) ? DY / SMALL : DY / TMP1;
            if (TMP2 < TMP3) TMP3 = TMP2;
        }
    ofr DT_tmp = o->p.cfl * TMP3;
    if (o->p.fixed_dt) {
        o->DT = o->p.dt_fixed;
        while (o->DT > DT_tmp) o->DT = o->DT / 2.0;
    } else {
        o->DT = DT_tmp;
    }
    o->TIME = o->TIME + o->DT;
}

/* ------------------------------------------------------------------------ */
/* 2nd-order masked central derivatives (derivatives.F:123-289), interior   */
/* ------------------------------------------------------------------------ */
static void d_x(ofw_ctx *o, const ofr *in, ofr *out) {
    const ofr DX = o->p.DX;
    OMP_FOR
    for (int J = o->Jbeg; J <= o->Jend; J++)
        for (int I = o->Ibeg; I <= o->Iend; I++)
            C2(out, I, J) = (C2(in, I + 1, J) - C2(in, I - 1, J)) / DX / 2.0 * (ofr)C2(o->MASK9, I, J);
}
static void d_y(ofw_ctx *o, const ofr *in, ofr *out) {
    const ofr DY = o->p.DY;
    OMP_FOR
    for (int J = o->Jbeg; J <= o->Jend; J++)
        for (int I = o->Ibeg; I <= o->Iend; I++)
            C2(out, I, J) = (C2(in, I, J + 1) - C2(in, I, J - 1)) / DY / 2.0 * (ofr)C2(o->MASK9, I, J);
}
static void d_xx(ofw_ctx *o, const ofr *in, ofr *out) {
    const ofr DX = o->p.DX;
    OMP_FOR
    for (int J = o->Jbeg; J <= o->Jend; J++)
        for (int I = o->Ibeg; I <= o->Iend; I++)
            C2(out, I, J) = (C2(in, I + 1, J) - 2.0 * C2(in, I, J) + C2(in, I - 1, J)) / DX / DX *
                            (ofr)C2(o->MASK9, I, J);
}
static void d_yy(ofw_ctx *o, const ofr *in, ofr *out) {
    const ofr DY = o->p.DY;
    OMP_FOR
    for (int J = o->Jbeg; J <= o->Jend; J++)
        for (int I = o->Ibeg; I <= o->Iend; I++)
            C2(out, I, J) = (C2(in, I, J + 1) - 2.0 * C2(in, I, J) + C2(in, I, J - 1)) / DY / DY *
                            (ofr)C2(o->MASK9, I, J);
}
static void d_xy(ofw_ctx *o, const ofr *in, ofr *out) {
    const ofr DX = o->p.DX, DY = o->p.DY;
    OMP_FOR
    for (int J = o->Jbeg; J <= o->Jend; J++)
        for (int I = o->Ibeg; I <= o->Iend; I++) {
            ofr t1 = (C2(in, I + 1, J + 1) - C2(in, I + 1, J - 1)) / 2.0 / DY;
            ofr t2 = (C2(in, I - 1, J + 1) - C2(in, I - 1, J - 1)) / 2.0 / DY;
            C2(out, I, J) = (t1 - t2) / 2.0 / DX * (ofr)C2(o->MASK9, I, J);
        }
}

/* ------------------------------------------------------------------------ */
/* CAL_DISPERSION (dispersion.F:62-506), CARTESIAN, DISP_TIME_LEFT = F      */
/* ------------------------------------------------------------------------ */
static void exchange_dispersion(ofw_ctx *o) {
    /* EXCHANGE_DISPERSION (bc.F:306-414), CARTESIAN, DISP_TIME_LEFT=F */
    phi_coll(o, o->Uxx, 2);
    phi_coll(o, o->DUxx, 2);
    phi_coll(o, o->Vyy, 3);
    phi_coll(o, o->DVyy, 3);
    phi_coll(o, o->Uxy, 1);
    phi_coll(o, o->DUxy, 1);
    phi_coll(o, o->Vxy, 1);
    phi_coll(o, o->DVxy, 1);
    if (o->p.gamma2 > ZERO) {
        phi_coll(o, o->Ut, 2);
        phi_coll(o, o->Vt, 3);
        phi_coll(o, o->Utx, 1);
        phi_coll(o, o->Vty, 1);
        phi_coll(o, o->Utxx, 2);
        phi_coll(o, o->Vtyy, 3);
        phi_coll(o, o->Utxy, 1);
        phi_coll(o, o->Vtxy, 1);
        phi_coll(o, o->DUtxx, 2);
        phi_coll(o, o->DVtyy, 3);
        phi_coll(o, o->DUtxy, 1);
        phi_coll(o, o->DVtxy, 1);
        phi_coll(o, o->Ux, 1);
        phi_coll(o, o->DUx, 1);
        phi_coll(o, o->Vy, 1);
        phi_coll(o, o->DVy, 1);
        phi_coll(o, o->Uy, 3);
        phi_coll(o, o->DUy, 3);
        phi_coll(o, o->Vx, 2);
        phi_coll(o, o->DVx, 2);
        phi_coll(o, o->ETAx, 2);
        phi_coll(o, o->ETAy, 3);
    }
}

void ofw_cal_dispersion(ofw_ctx *o) {
    const int M = o->Mloc, N = o->Nloc;
    const size_t nc = (size_t)M * N;
    const ofr DX = o->p.DX, DY = o->p.DY, mdf = o->p.min_depth_frc;
    const ofr gamma2 = o->p.gamma2;
    const ofr Beta_1 = o->Beta_1, Beta_2 = o->Beta_2, b2 = o->b2;
    ofr *DU = (ofr *)calloc(nc, sizeof(ofr));
    ofr *DV = (ofr *)calloc(nc, sizeof(ofr));
    ofr *DUt = (ofr *)calloc(nc, sizeof(ofr));
    ofr *DVt = (ofr *)calloc(nc, sizeof(ofr));

    d_xx(o, o->U, o->Uxx);
    d_xy(o, o->U, o->Uxy);
    d_xy(o, o->V, o->Vxy);
    d_yy(o, o->V, o->Vyy);
    if (gamma2 > ZERO) {
        d_x(o, o->U, o->Ux);
        d_x(o, o->V, o->Vx);
        d_y(o, o->U, o->Uy);
        d_y(o, o->V, o->Vy);
        d_x(o, o->Eta, o->ETAx);
        d_y(o, o->Eta, o->ETAy);
    } else if (o->p.show_breaking) {
        d_x(o, o->Eta, o->ETAx);
        d_y(o, o->Eta, o->ETAy);
    }
    /* dispersion.F:103-119 */
    OMP_FOR
    for (int J = 1; J <= N - 1; J++)
        for (int I = 1; I <= M - 1; I++) {
            C2(DU, I, J) = dmax(C2(o->Depth, I, J), mdf) * C2(o->U, I, J);
            C2(DV, I, J) = dmax(C2(o->Depth, I, J), mdf) * C2(o->V, I, J);
            C2(o->ETAT, I, J) = -(X2(o->P, I + 1, J) - X2(o->P, I, J)) / DX -
                                (Y2(o->Q, I, J + 1) - Y2(o->Q, I, J)) / DY;
        }
    if (gamma2 > ZERO) {
        OMP_FOR
        for (int J = 1; J <= N; J++)
            for (int I = 1; I <= M; I++) {
                C2(o->Ut, I, J) = (C2(o->U, I, J) - C2(o->U0, I, J)) / o->DT;
                C2(o->Vt, I, J) = (C2(o->V, I, J) - C2(o->V0, I, J)) / o->DT;
                C2(DUt, I, J) = dmax(C2(o->Depth, I, J), mdf) * C2(o->Ut, I, J);
                C2(DVt, I, J) = dmax(C2(o->Depth, I, J), mdf) * C2(o->Vt, I, J);
            }
    }
    d_xx(o, DU, o->DUxx);
    d_xy(o, DU, o->DUxy);
    d_xy(o, DV, o->DVxy);
    d_yy(o, DV, o->DVyy);
    if (gamma2 > ZERO) {
        d_x(o, DU, o->DUx);
        d_x(o, DV, o->DVx);
        d_y(o, DU, o->DUy);
        d_y(o, DV, o->DVy);
        d_x(o, o->Ut, o->Utx);
        d_y(o, o->Vt, o->Vty);
        d_xx(o, o->Ut, o->Utxx);
        d_yy(o, o->Vt, o->Vtyy);
        d_xy(o, o->Ut, o->Utxy);
        d_xy(o, o->Vt, o->Vtxy);
        d_x(o, DUt, o->DUtx);
        d_y(o, DVt, o->DVty);
        d_xx(o, DUt, o->DUtxx);
        d_yy(o, DVt, o->DVtyy);
        d_xy(o, DUt, o->DUtxy);
        d_xy(o, DVt, o->DVtxy);
    }
    /* wall rows of the cross derivatives (dispersion.F:189-286) */
    ofr *cross[8] = {o->Uxy, o->DUxy, o->Vxy, o->DVxy, o->Utxy, o->DUtxy, o->Vtxy, o->DVtxy};
    for (int k = 0; k < 8; k++) {
        for (int J = 1; J <= N; J++) C2(cross[k], o->Ibeg, J) = ZERO;
        for (int J = 1; J <= N; J++) C2(cross[k], o->Iend, J) = ZERO;
        for (int I = 1; I <= M; I++) C2(cross[k], I, o->Jbeg) = ZERO;
        for (int I = 1; I <= M; I++) C2(cross[k], I, o->Jend) = ZERO;
    }
    exchange_dispersion(o);

    /* U4, V4, U1p, V1p over all cells (dispersion.F:293-384) */
    const ofr c4a = 1.0 / 3.0 - Beta_1 + 0.5 * Beta_1 * Beta_1;
    OMP_FOR
    for (int J = 1; J <= N; J++)
        for (int I = 1; I <= M; I++) {
            ofr D = C2(o->Depth, I, J);
            C2(o->U4, I, J) = (1.0 / 3.0 - Beta_1 + 0.5 * Beta_1 * Beta_1) * D * D *
                                  (C2(o->Uxx, I, J) + C2(o->Vxy, I, J)) +
                              (Beta_1 - 1.0 / 2.0) * D * (C2(o->DUxx, I, J) + C2(o->DVxy, I, J));
            C2(o->V4, I, J) = (1.0 / 3.0 - Beta_1 + 0.5 * Beta_1 * Beta_1) * D * D *
                                  (C2(o->Uxy, I, J) + C2(o->Vyy, I, J)) +
                              (Beta_1 - 1.0 / 2.0) * D * (C2(o->DUxy, I, J) + C2(o->DVyy, I, J));
            if (gamma2 > ZERO) {
                ofr UxxVxy = C2(o->Uxx, I, J) + C2(o->Vxy, I, J);
                ofr UxyVyy = C2(o->Uxy, I, J) + C2(o->Vyy, I, J);
                ofr HUxxHVxy = C2(o->DUxx, I, J) + C2(o->DVxy, I, J);
                ofr HUxyHVyy = C2(o->DUxy, I, J) + C2(o->DVyy, I, J);
                ofr rh = D, reta = C2(o->Eta, I, J);
                ofr ken1 = (1.0 / 6.0 - Beta_1 + Beta_1 * Beta_1) * rh * reta * Beta_2 +
                              (1.0 / 2.0 * Beta_1 * Beta_1 - 1.0 / 6.0) * reta * reta * Beta_2 * Beta_2;
                ofr ken2 = (Beta_1 - 1.0 / 2.0) * reta * Beta_2;
                ofr m9 = (ofr)C2(o->MASK9, I, J);
                C2(o->U4, I, J) = C2(o->U4, I, J) + gamma2 * m9 * (ken1 * UxxVxy + ken2 * HUxxHVxy);
                C2(o->V4, I, J) = C2(o->V4, I, J) + gamma2 * m9 * (ken1 * UxyVyy + ken2 * HUxyHVyy);
            }
            C2(o->U1p, I, J) = 0.5 * (1.0 - Beta_1) * (1.0 - Beta_1) * D * D *
                                   (C2(o->Uxx, I, J) + C2(o->Vxy, I, J)) +
                               (Beta_1 - 1.0) * D * (C2(o->DUxx, I, J) + C2(o->DVxy, I, J));
            C2(o->V1p, I, J) = 0.5 * (1.0 - Beta_1) * (1.0 - Beta_1) * D * D *
                                   (C2(o->Uxy, I, J) + C2(o->Vyy, I, J)) +
                               (Beta_1 - 1.0) * D * (C2(o->DUxy, I, J) + C2(o->DVyy, I, J));
        }
    (void)c4a;

    /* gamma2 terms, interior (dispersion.F:399-503) */
    if (gamma2 > ZERO) {
        OMP_FOR
        for (int J = o->Jbeg; J <= o->Jend; J++)
            for (int I = o->Ibeg; I <= o->Iend; I++) {
                ofr UxxVxy = C2(o->Uxx, I, J) + C2(o->Vxy, I, J);
                ofr UxyVyy = C2(o->Uxy, I, J) + C2(o->Vyy, I, J);
                ofr UxxVxy_x = (C2(o->Uxx, I + 1, J) + C2(o->Vxy, I + 1, J) - C2(o->Uxx, I - 1, J) -
                                   C2(o->Vxy, I - 1, J)) / 2.0 / DX;
                ofr UxxVxy_y = (C2(o->Uxx, I, J + 1) + C2(o->Vxy, I, J + 1) - C2(o->Uxx, I, J - 1) -
                                   C2(o->Vxy, I, J - 1)) / 2.0 / DY;
                ofr UxyVyy_x = (C2(o->Uxy, I + 1, J) + C2(o->Vyy, I + 1, J) - C2(o->Uxy, I - 1, J) -
                                   C2(o->Vyy, I - 1, J)) / 2.0 / DX;
                ofr UxyVyy_y = (C2(o->Uxy, I, J + 1) + C2(o->Vyy, I, J + 1) - C2(o->Uxy, I, J - 1) -
                                   C2(o->Vyy, I, J - 1)) / 2.0 / DY;
                ofr HUxxHVxy = C2(o->DUxx, I, J) + C2(o->DVxy, I, J);
                ofr HUxyHVyy = C2(o->DUxy, I, J) + C2(o->DVyy, I, J);
                ofr HUxxHVxy_x = (C2(o->DUxx, I + 1, J) + C2(o->DVxy, I + 1, J) -
                                     C2(o->DUxx, I - 1, J) - C2(o->DVxy, I - 1, J)) / 2.0 / DX;
                ofr HUxxHVxy_y = (C2(o->DUxx, I, J + 1) + C2(o->DVxy, I, J + 1) -
                                     C2(o->DUxx, I, J - 1) - C2(o->DVxy, I, J - 1)) / 2.0 / DY;
                ofr HUxyHVyy_x = (C2(o->DUxy, I + 1, J) + C2(o->DVyy, I + 1, J) -
                                     C2(o->DUxy, I - 1, J) - C2(o->DVyy, I - 1, J)) / 2.0 / DX;
                ofr HUxyHVyy_y = (C2(o->DUxy, I, J + 1) + C2(o->DVyy, I, J + 1) -
                                     C2(o->DUxy, I, J - 1) - C2(o->DVyy, I, J - 1)) / 2.0 / DY;
                ofr rh = C2(o->Depth, I, J);
                ofr rhx = (C2(o->Depth, I + 1, J) - C2(o->Depth, I - 1, J)) / 2.0 / DX;
                ofr rhy = (C2(o->Depth, I, J + 1) - C2(o->Depth, I, J - 1)) / 2.0 / DY;
                ofr reta = C2(o->Eta, I, J);
                ofr ETAx = C2(o->ETAx, I, J), ETAy = C2(o->ETAy, I, J), ETAT = C2(o->ETAT, I, J);
                ofr Utx = C2(o->Utx, I, J), Vty = C2(o->Vty, I, J);
                ofr U1pp = -reta * Beta_2 * ETAx * Beta_2 * (Utx + Vty) -
                              0.5 * reta * reta * Beta_2 * Beta_2 * (C2(o->Utxx, I, J) + C2(o->Vtxy, I, J)) -
                              ETAx * Beta_2 * (C2(o->DUtx, I, J) + C2(o->DVty, I, J)) -
                              reta * Beta_2 * (C2(o->DUtxx, I, J) + C2(o->DVtxy, I, J));
                ofr V1pp = -reta * Beta_2 * ETAy * Beta_2 * (Utx + Vty) -
                              0.5 * reta * reta * Beta_2 * Beta_2 * (C2(o->Utxy, I, J) + C2(o->Vtyy, I, J)) -
                              ETAy * Beta_2 * (C2(o->DUtx, I, J) + C2(o->DVty, I, J)) -
                              reta * Beta_2 * (C2(o->DUtxy, I, J) + C2(o->DVtyy, I, J));
                ofr ken1 = Beta_1 * (1.0 - Beta_1) * rh * ETAT * Beta_2 -
                              Beta_1 * Beta_1 * reta * Beta_2 * ETAT * Beta_2;
                ofr ken2 = Beta_1 * (1.0 - Beta_1) * rh * reta * Beta_2 -
                              0.5 * Beta_1 * Beta_1 * reta * reta * Beta_2 * Beta_2;
                ofr ken3 = Beta_1 * ETAT * Beta_2;
                ofr ken4 = Beta_1 * reta * Beta_2;
                U1pp = U1pp - ken1 * UxxVxy - ken2 * (C2(o->Utxx, I, J) + C2(o->Vtxy, I, J)) +
                       ken3 * HUxxHVxy + ken4 * (C2(o->DUtxx, I, J) + C2(o->DVtxy, I, J));
                V1pp = V1pp - ken1 * UxyVyy - ken2 * (C2(o->Utxy, I, J) + C2(o->Vtyy, I, J)) +
                       ken3 * HUxyHVyy + ken4 * (C2(o->DUtxy, I, J) + C2(o->DVtyy, I, J));
                C2(o->U1pp, I, J) = U1pp;
                C2(o->V1pp, I, J) = V1pp;

                ofr Ux = C2(o->Ux, I, J), Vx = C2(o->Vx, I, J), Uy = C2(o->Uy, I, J),
                       Vy = C2(o->Vy, I, J);
                ofr DUx = C2(o->DUx, I, J), DVy = C2(o->DVy, I, J);
                ofr Uc = C2(o->U, I, J), Vc = C2(o->V, I, J);
                ken1 = (Beta_1 - 1.0) * (rhx + ETAx) * Beta_2;
                ken2 = (Beta_1 - 1.0) * (rh + reta) * Beta_2;
                ken3 = ((1.0 - Beta_1) * (1.0 - Beta_1) * rh * rhx * Beta_2 * Beta_2 -
                        Beta_1 * (1.0 - Beta_1) * (rhx * reta * Beta_2 + rh * ETAx * Beta_2) +
                        (Beta_1 * Beta_1 - 1.0) * reta * ETAx * Beta_2 * Beta_2);
                ken4 = (0.5 * (1.0 - Beta_1) * (1.0 - Beta_1) * rh * rh * Beta_2 * Beta_2 -
                        Beta_1 * (1.0 - Beta_1) * rh * reta * Beta_2 +
                        0.5 * (Beta_1 * Beta_1 - 1.0) * reta * reta * Beta_2 * Beta_2);
                ofr ken5 = ((1.0 - Beta_1) * (1.0 - Beta_1) * rh * rhy * Beta_2 * Beta_2 -
                               Beta_1 * (1.0 - Beta_1) * (rhy * reta * Beta_2 + rh * ETAy * Beta_2) +
                               (Beta_1 * Beta_1 - 1.0) * reta * ETAy * Beta_2 * Beta_2);
                C2(o->U2, I, J) =
                    ken1 * (Uc * HUxxHVxy + Vc * HUxyHVyy) +
                    ken2 * (Ux * HUxxHVxy + Uc * HUxxHVxy_x + Vx * HUxyHVyy + Vc * HUxyHVyy_x) +
                    ken3 * (Uc * UxxVxy + Vc * UxyVyy) +
                    ken4 * (Ux * UxxVxy + Uc * UxxVxy_x + Vx * UxyVyy + Vc * UxyVyy_x) +
                    Beta_2 * Beta_2 * (DUx + DVy + reta * Beta_2 * (Ux + Vy)) *
                        (HUxxHVxy + ETAx * Beta_2 * (Ux + Vy) + reta * Beta_2 * UxxVxy);
                ken1 = (Beta_1 - 1.0) * (rhy + ETAy) * Beta_2;
                C2(o->V2, I, J) =
                    ken1 * (Uc * HUxxHVxy + Vc * HUxyHVyy) +
                    ken2 * (Uy * HUxxHVxy + Uc * HUxxHVxy_y + Vy * HUxyHVyy + Vc * HUxyHVyy_y) +
                    ken5 * (Uc * UxxVxy + Vc * UxyVyy) +
                    ken4 * (Uy * UxxVxy + Uc * UxxVxy_y + Vy * UxyVyy + Vc * UxyVyy_y) +
                    Beta_2 * Beta_2 * (DUx + DVy + reta * Beta_2 * (Ux + Vy)) *
                        (HUxyHVyy + ETAy * Beta_2 * (Ux + Vy) + reta * Beta_2 * UxyVyy);
                ofr omega_0 = Vx - Uy;
                ofr omega_1 = (b2 * rhx + Beta_1 * ETAx) * Beta_2 *
                                     (HUxyHVyy + (b2 * rh + Beta_1 * reta) * Beta_2 * UxyVyy) -
                                 (b2 * rhy + Beta_1 * ETAy) * Beta_2 *
                                     (HUxxHVxy + (b2 * rh + Beta_1 * reta) * Beta_2 * UxxVxy);
                ken1 = ((Beta_1 - 1.0 / 2.0) * (reta + rh) * Beta_2);
                ken2 = (1.0 / 3.0 - Beta_1 + 0.5 * Beta_1 * Beta_1) * rh * rh * Beta_2 * Beta_2 +
                       (1.0 / 6.0 - Beta_1 + Beta_1 * Beta_1) * rh * reta * Beta_2 +
                       (1.0 / 2.0 * Beta_1 * Beta_1 - 1.0 / 6.0) * reta * reta * Beta_2 * Beta_2;
                C2(o->U3, I, J) = -Vc * omega_1 - omega_0 * (ken1 * HUxyHVyy + ken2 * UxyVyy);
                C2(o->V3, I, J) = Uc * omega_1 + omega_0 * (ken1 * HUxxHVxy + ken2 * UxxVxy);
            }
    }
    free(DU);
    free(DV);
    free(DUt);
    free(DVt);
}

/* ------------------------------------------------------------------------ */
/* FLUXES (fluxes.F:52-117): CONSTRUCTION_HO + WAVE_SPEED + HLL + BC        */
/* ------------------------------------------------------------------------ */

/* 3-argument minmod-like limiter of CONSTRUCT_HO_X (fluxes.F:1552-1566) */
static inline ofr lim3(ofr a, ofr b, ofr c) {
    if (a >= 0.0) return dmax(0.0, min3(a, 2.0 * b, 2.0 * c));
    return dmin(0.0, max3(a, 2.0 * b, 2.0 * c));
}

/* Din for one position: v[0..3] = Vin(i-2..i+1), m[0..3] = MASK(i-2..i+1).
 * fluxes.F:1548-1598 */
static inline ofr ho_din(const ofr *v, const int *m) {
    ofr TXP1 = v[1] - v[0];
    ofr TXP2 = v[2] - v[1];
    ofr TXP3 = v[3] - v[2];
    ofr DVP1 = lim3(TXP1, TXP2, TXP3);
    ofr DVP2 = lim3(TXP2, TXP3, TXP1);
    ofr DVP3 = lim3(TXP3, TXP1, TXP2);
    if (m[0] == 0 || m[3] == 0) {
        TXP2 = v[2] - v[1];
        TXP1 = TXP2;
        TXP3 = TXP2;
        DVP1 = lim3(TXP1, TXP2, TXP3);
        DVP2 = lim3(TXP2, TXP3, TXP1);
        DVP3 = lim3(TXP3, TXP1, TXP2);
    }
    if (m[1] == 0 || m[2] == 0) {
        DVP1 = ZERO;
        DVP2 = ZERO;
        DVP3 = ZERO;
    }
    return TXP2 - 1.0 / 6.0 * (DVP3 - 2.0 * DVP2 + DVP1);
}

/* van Leer face values (fluxes.F:1602-1630): returns OutL at face i from
 * Din(i-1), Din(i) and Vin(i-1); OutR from Din(i), Din(i+1) and Vin(i). */
static inline ofr vl_guard(ofr t) {
    if (fabs(t) <= SMALL) t = SMALL * copysign(1.0, t);
    return t;
}
static inline ofr vl_phi(ofr rat) {
    ofr van = 0.0;
    if (fabs(1.0 + rat) > SMALL) van = (rat + fabs(rat)) / (1.0 + rat);
    return van;
}
static inline ofr ho_left(ofr vim1, ofr d0, ofr d1) {
    ofr TMP1 = vl_guard(d0), TMP2 = vl_guard(d1);
    ofr VAN1 = vl_phi(TMP2 / TMP1);
    ofr VAN2 = vl_phi(TMP1 / TMP2);
    return vim1 + (1.0 / 6.0) * (VAN1 * TMP1 + 2.0 * VAN2 * TMP2);
}
static inline ofr ho_right(ofr vi, ofr d0, ofr d1) {
    ofr TMP1 = vl_guard(d0), TMP2 = vl_guard(d1);
    ofr VAN1 = vl_phi(TMP2 / TMP1);
    ofr VAN2 = vl_phi(TMP1 / TMP2);
    return vi - (1.0 / 6.0) * (2.0 * VAN1 * TMP1 + VAN2 * TMP2);
}

/* CONSTRUCT_HO_X (fluxes.F:1531-1639) */
static void construct_ho_x(ofw_ctx *o, const ofr *Vin, ofr *OutL, ofr *OutR) {
    const int Ib = o->Ibeg, Ie = o->Iend, M = o->Mloc;
    OMP_FOR
    for (int J = o->Jbeg; J <= o->Jend; J++) {
        ofr *Din = (ofr *)calloc((size_t)M + 1, sizeof(ofr));
        for (int I = Ib - 1; I <= Ie + 2; I++) {
            ofr v[4];
            int m[4];
            for (int k = 0; k < 4; k++) {
                v[k] = C2(Vin, I - 2 + k, J);
                m[k] = C2(o->MASK, I - 2 + k, J);
            }
            Din[I] = ho_din(v, m);
        }
        for (int I = Ib; I <= Ie + 1; I++) {
            X2(OutL, I, J) = ho_left(C2(Vin, I - 1, J), Din[I - 1], Din[I]);
            X2(OutR, I, J) = ho_right(C2(Vin, I, J), Din[I], Din[I + 1]);
        }
        free(Din);
    }
}

/* CONSTRUCT_HO_Y (fluxes.F:1646-1754) */
static void construct_ho_y(ofw_ctx *o, const ofr *Vin, ofr *OutL, ofr *OutR) {
    const int Jb = o->Jbeg, Je = o->Jend, N = o->Nloc;
    OMP_FOR
    for (int I = o->Ibeg; I <= o->Iend; I++) {
        ofr *Din = (ofr *)calloc((size_t)N + 1, sizeof(ofr));
        for (int J = Jb - 1; J <= Je + 2; J++) {
            ofr v[4];
            int m[4];
            for (int k = 0; k < 4; k++) {
                v[k] = C2(Vin, I, J - 2 + k);
                m[k] = C2(o->MASK, I, J - 2 + k);
            }
            Din[J] = ho_din(v, m);
        }
        for (int J = Jb; J <= Je + 1; J++) {
            Y2(OutL, I, J) = ho_left(C2(Vin, I, J - 1), Din[J - 1], Din[J]);
            Y2(OutR, I, J) = ho_right(C2(Vin, I, J), Din[J], Din[J + 1]);
        }
        free(Din);
    }
}

/* CONSTRUCTION_HO (fluxes.F:1324-1524), CARTESIAN, DISPERSION */
static void construction_ho(ofw_ctx *o) {
    const int M = o->Mloc, N = o->Nloc, M1 = o->Mloc1, N1 = o->Nloc1;
    const ofr g1 = o->p.gamma1, g3 = o->p.gamma3;
    construct_ho_x(o, o->U, o->UxL, o->UxR);
    construct_ho_x(o, o->V, o->VxL, o->VxR);
    construct_ho_x(o, o->HU, o->HUxL, o->HUxR);
    construct_ho_x(o, o->HV, o->HVxL, o->HVxR);
    construct_ho_x(o, o->Eta, o->EtaRxL, o->EtaRxR);
    OMP_FOR
    for (int J = 1; J <= N; J++)
        for (int I = 1; I <= M1; I++) {
            X2(o->HxL, I, J) = X2(o->EtaRxL, I, J) + X2(o->Depthx, I, J);
            X2(o->HxR, I, J) = X2(o->EtaRxR, I, J) + X2(o->Depthx, I, J);
        }
    if (o->p.dispersion) {
        construct_ho_x(o, o->U4, o->U4xL, o->U4xR);
        construct_ho_x(o, o->V4, o->V4xL, o->V4xR);
    }
    OMP_FOR
    for (int J = 1; J <= N; J++)
        for (int I = 1; I <= M1; I++) {
            /* MASK9u(Mloc1,:) = MASK9(Mloc,:) (fluxes.F:1333) */
            ofr m9 = (ofr)C2(o->MASK9, I <= M ? I : M, J);
            ofr EL = X2(o->EtaRxL, I, J), ER = X2(o->EtaRxR, I, J), Dx = X2(o->Depthx, I, J);
            X2(o->PL, I, J) = X2(o->HUxL, I, J) + g1 * m9 * X2(o->HxL, I, J) * X2(o->U4xL, I, J);
            X2(o->PR, I, J) = X2(o->HUxR, I, J) + g1 * m9 * X2(o->HxR, I, J) * X2(o->U4xR, I, J);
            X2(o->FxL, I, J) = g3 * X2(o->PL, I, J) * (X2(o->UxL, I, J) + g1 * m9 * X2(o->U4xL, I, J)) +
                               0.5 * GRAV * ((EL) * (EL)*g3 + 2.0 * (EL) * (Dx));
            X2(o->FxR, I, J) = g3 * X2(o->PR, I, J) * (X2(o->UxR, I, J) + g1 * m9 * X2(o->U4xR, I, J)) +
                               0.5 * GRAV * ((ER) * (ER)*g3 + 2.0 * (ER) * (Dx));
            X2(o->GxL, I, J) = X2(o->HxL, I, J) * (X2(o->UxL, I, J) + g1 * m9 * X2(o->U4xL, I, J)) *
                               (X2(o->VxL, I, J) + g1 * m9 * X2(o->V4xL, I, J)) * g3;
            X2(o->GxR, I, J) = X2(o->HxR, I, J) * (X2(o->UxR, I, J) + g1 * m9 * X2(o->U4xR, I, J)) *
                               (X2(o->VxR, I, J) + g1 * m9 * X2(o->V4xR, I, J)) * g3;
        }
    construct_ho_y(o, o->U, o->UyL, o->UyR);
    construct_ho_y(o, o->V, o->VyL, o->VyR);
    construct_ho_y(o, o->HV, o->HVyL, o->HVyR);
    construct_ho_y(o, o->HU, o->HUyL, o->HUyR);
    construct_ho_y(o, o->Eta, o->EtaRyL, o->EtaRyR);
    OMP_FOR
    for (int J = 1; J <= N1; J++)
        for (int I = 1; I <= M; I++) {
            Y2(o->HyL, I, J) = Y2(o->EtaRyL, I, J) + Y2(o->Depthy, I, J);
            Y2(o->HyR, I, J) = Y2(o->EtaRyR, I, J) + Y2(o->Depthy, I, J);
        }
    if (o->p.dispersion) {
        construct_ho_y(o, o->V4, o->V4yL, o->V4yR);
        construct_ho_y(o, o->U4, o->U4yL, o->U4yR);
    }
    OMP_FOR
    for (int J = 1; J <= N1; J++)
        for (int I = 1; I <= M; I++) {
            ofr m9 = (ofr)C2(o->MASK9, I, J <= N ? J : N);
            ofr EL = Y2(o->EtaRyL, I, J), ER = Y2(o->EtaRyR, I, J), Dy = Y2(o->Depthy, I, J);
            Y2(o->QL, I, J) = Y2(o->HVyL, I, J) + g1 * m9 * Y2(o->HyL, I, J) * Y2(o->V4yL, I, J);
            Y2(o->QR, I, J) = Y2(o->HVyR, I, J) + g1 * m9 * Y2(o->HyR, I, J) * Y2(o->V4yR, I, J);
            Y2(o->GyL, I, J) = g3 * Y2(o->QL, I, J) * (Y2(o->VyL, I, J) + g1 * m9 * Y2(o->V4yL, I, J)) +
                               0.5 * GRAV * ((EL) * (EL)*g3 + 2.0 * (EL) * (Dy));
            Y2(o->GyR, I, J) = g3 * Y2(o->QR, I, J) * (Y2(o->VyR, I, J) + g1 * m9 * Y2(o->V4yR, I, J)) +
                               0.5 * GRAV * ((ER) * (ER)*g3 + 2.0 * (ER) * (Dy));
            Y2(o->FyL, I, J) = Y2(o->HyL, I, J) * (Y2(o->UyL, I, J) + g1 * m9 * Y2(o->U4yL, I, J)) *
                               (Y2(o->VyL, I, J) + g1 * m9 * Y2(o->V4yL, I, J)) * g3;
            Y2(o->FyR, I, J) = Y2(o->HyR, I, J) * (Y2(o->UyR, I, J) + g1 * m9 * Y2(o->U4yR, I, J)) *
                               (Y2(o->VyR, I, J) + g1 * m9 * Y2(o->V4yR, I, J)) * g3;
        }
}

/* WAVE_SPEED (fluxes.F:352-439) */
static void wave_speed(ofw_ctx *o) {
    const int M = o->Mloc, N = o->Nloc, M1 = o->Mloc1, N1 = o->Nloc1;
    OMP_FOR
    for (int J = 1 + NGHOST; J <= N - NGHOST; J++)
        for (int I = 1 + NGHOST; I <= M1 - NGHOST; I++) {
            ofr UL = X2(o->UxL, I, J), UR = X2(o->UxR, I, J);
            ofr SQR_PHI_L = sqrt(GRAV * fabs(X2(o->HxL, I, J)));
            ofr SQR_PHI_R = sqrt(GRAV * fabs(X2(o->HxR, I, J)));
            ofr SQR_PHI_S = 0.5 * (SQR_PHI_L + SQR_PHI_R) + 0.25 * (UL - UR);
            ofr U_S = 0.5 * (UL + UR) + SQR_PHI_L - SQR_PHI_R;
            X2(o->SxL, I, J) = dmin(UL - SQR_PHI_L, U_S - SQR_PHI_S);
            X2(o->SxR, I, J) = dmax(UR + SQR_PHI_R, U_S + SQR_PHI_S);
        }
    for (int J = 1 + NGHOST; J <= N - NGHOST; J++) {
        for (int I = 1; I <= NGHOST; I++) {
            X2(o->SxL, I, J) = X2(o->SxL, NGHOST + 1, J);
            X2(o->SxR, I, J) = X2(o->SxR, NGHOST + 1, J);
        }
        for (int I = M1 - NGHOST + 1; I <= M1; I++) {
            X2(o->SxL, I, J) = X2(o->SxL, M1 - NGHOST, J);
            X2(o->SxR, I, J) = X2(o->SxR, M1 - NGHOST, J);
        }
    }
    for (int I = 1; I <= M1; I++) {
        for (int J = 1; J <= NGHOST; J++) {
            X2(o->SxL, I, J) = X2(o->SxL, I, NGHOST + 1);
            X2(o->SxR, I, J) = X2(o->SxR, I, NGHOST + 1);
        }
        for (int J = N - NGHOST + 1; J <= N; J++) {
            X2(o->SxL, I, J) = X2(o->SxL, I, N - NGHOST);
            X2(o->SxR, I, J) = X2(o->SxR, I, N - NGHOST);
        }
    }
    OMP_FOR
    for (int J = 1 + NGHOST; J <= N1 - NGHOST; J++)
        for (int I = 1 + NGHOST; I <= M - NGHOST; I++) {
            ofr VL = Y2(o->VyL, I, J), VR = Y2(o->VyR, I, J);
            ofr SQR_PHI_L = sqrt(GRAV * fabs(Y2(o->HyL, I, J)));
            ofr SQR_PHI_R = sqrt(GRAV * fabs(Y2(o->HyR, I, J)));
            ofr SQR_PHI_S = 0.5 * (SQR_PHI_L + SQR_PHI_R) + 0.25 * (VL - VR);
            ofr U_S = 0.5 * (VL + VR) + SQR_PHI_L - SQR_PHI_R;
            Y2(o->SyL, I, J) = dmin(VL - SQR_PHI_L, U_S - SQR_PHI_S);
            Y2(o->SyR, I, J) = dmax(VR + SQR_PHI_R, U_S + SQR_PHI_S);
        }
    for (int I = 1 + NGHOST; I <= M - NGHOST; I++) {
        for (int J = 1; J <= NGHOST; J++) {
            Y2(o->SyL, I, J) = Y2(o->SyL, I, NGHOST + 1);
            Y2(o->SyR, I, J) = Y2(o->SyR, I, NGHOST + 1);
        }
        for (int J = N1 - NGHOST + 1; J <= N1; J++) {
            Y2(o->SyL, I, J) = Y2(o->SyL, I, N1 - NGHOST);
            Y2(o->SyR, I, J) = Y2(o->SyR, I, N1 - NGHOST);
        }
    }
    for (int J = 1; J <= N1; J++) {
        for (int I = 1; I <= NGHOST; I++) {
            Y2(o->SyL, I, J) = Y2(o->SyL, NGHOST + 1, J);
            Y2(o->SyR, I, J) = Y2(o->SyR, NGHOST + 1, J);
        }
        for (int I = M - NGHOST + 1; I <= M; I++) {
            Y2(o->SyL, I, J) = Y2(o->SyL, M - NGHOST, J);
            Y2(o->SyR, I, J) = Y2(o->SyR, M - NGHOST, J);
        }
    }
}

/* HLL (fluxes.F:171-194) on a whole array of n entries */
static void hll(size_t n, const ofr *SL, const ofr *SR, const ofr *FL, const ofr *FR,
                const ofr *UL, const ofr *UR, ofr *FOUT) {
    OMP_FOR
    for (size_t k = 0; k < n; k++) {
        if (SL[k] >= ZERO) {
            FOUT[k] = FL[k];
        } else if (SR[k] <= ZERO) {
            FOUT[k] = FR[k];
        } else {
            ofr f = SR[k] * FL[k] - SL[k] * FR[k] + SL[k] * SR[k] * (UR[k] - UL[k]);
            if (fabs(SR[k] - SL[k]) < SMALL) f = f / SMALL;
            else f = f / (SR[k] - SL[k]);
            FOUT[k] = f;
        }
    }
}

/* BOUNDARY_CONDITION (bc.F:53-295), serial, no ABS/LEFT_BC_IRR/COUPLING */
static void boundary_condition(ofw_ctx *o) {
    const ofr g3 = o->p.gamma3;
    const int Ib = o->Ibeg, Ie = o->Iend, Jb = o->Jbeg, Je = o->Jend;
#define PRESS(Xi, Deps) (0.5 * GRAV * ((Xi) * (Xi)*g3 + 2.0 * (Xi) * (Deps)))
    for (int J = Jb; J <= Je; J++) {
        X2(o->P, Ib, J) = ZERO;
        X2(o->Fx, Ib, J) = PRESS(X2(o->EtaRxR, Ib, J), X2(o->Depthx, Ib, J));
        X2(o->Gx, Ib, J) = ZERO;
    }
    for (int J = Jb; J <= Je; J++) {
        X2(o->P, o->Iend1, J) = ZERO;
        X2(o->Fx, o->Iend1, J) = PRESS(X2(o->EtaRxL, o->Iend1, J), X2(o->Depthx, o->Iend1, J));
        X2(o->Gx, o->Iend1, J) = ZERO;
    }
    if (!o->p.periodic) {
        for (int I = Ib; I <= Ie; I++) {
            Y2(o->Q, I, Jb) = ZERO;
            Y2(o->Fy, I, Jb) = ZERO;
            Y2(o->Gy, I, Jb) = PRESS(Y2(o->EtaRyR, I, Jb), Y2(o->Depthy, I, Jb));
        }
        for (int I = Ib; I <= Ie; I++) {
            Y2(o->Q, I, o->Jend1) = ZERO;
            Y2(o->Fy, I, o->Jend1) = ZERO;
            Y2(o->Gy, I, o->Jend1) = PRESS(Y2(o->EtaRyL, I, o->Jend1), Y2(o->Depthy, I, o->Jend1));
        }
    }
    for (int J = Jb - 1; J <= Je + 1; J++)
        for (int I = Ib - 1; I <= Ie + 1; I++) {
            if (C2(o->MASK, I, J) < 1) {
                X2(o->P, I, J) = ZERO;
                if (I != Ib)
                    X2(o->Fx, I, J) = PRESS(X2(o->EtaRxL, I, J), X2(o->Depthx, I, J)) * (ofr)C2(o->MASK, I - 1, J);
                else
                    X2(o->Fx, I, J) = ZERO;
                X2(o->Gx, I, J) = ZERO;
                X2(o->P, I + 1, J) = ZERO;
                if (I != Ie)
                    X2(o->Fx, I + 1, J) =
                        PRESS(X2(o->EtaRxR, I + 1, J), X2(o->Depthx, I + 1, J)) * (ofr)C2(o->MASK, I + 1, J);
                else
                    X2(o->Fx, I + 1, J) = ZERO;
                X2(o->Gx, I + 1, J) = ZERO;
                Y2(o->Q, I, J) = ZERO;
                Y2(o->Fy, I, J) = ZERO;
                if (J != Jb)
                    Y2(o->Gy, I, J) = PRESS(Y2(o->EtaRyL, I, J), Y2(o->Depthy, I, J)) * (ofr)C2(o->MASK, I, J - 1);
                else
                    Y2(o->Gy, I, J) = ZERO;
                Y2(o->Q, I, J + 1) = ZERO;
                Y2(o->Fy, I, J + 1) = ZERO;
                if (J != Je)
                    Y2(o->Gy, I, J + 1) =
                        PRESS(Y2(o->EtaRyR, I, J + 1), Y2(o->Depthy, I, J + 1)) * (ofr)C2(o->MASK, I, J + 1);
                else
                    Y2(o->Gy, I, J + 1) = ZERO;
            }
        }
#undef PRESS
}

void ofw_fluxes(ofw_ctx *o) {
    construction_ho(o);
    wave_speed(o);
    const size_t nx = (size_t)o->Mloc1 * o->Nloc, ny = (size_t)o->Mloc * o->Nloc1;
    /* FLUX_AT_INTERFACE_HLL (fluxes.F:150-161) */
    hll(nx, o->SxL, o->SxR, o->PL, o->PR, o->EtaRxL, o->EtaRxR, o->P);
    hll(ny, o->SyL, o->SyR, o->QL, o->QR, o->EtaRyL, o->EtaRyR, o->Q);
    hll(nx, o->SxL, o->SxR, o->FxL, o->FxR, o->HUxL, o->HUxR, o->Fx);
    hll(ny, o->SyL, o->SyR, o->FyL, o->FyR, o->HUyL, o->HUyR, o->Fy);
    hll(nx, o->SxL, o->SxR, o->GxL, o->GxR, o->HVxL, o->HVxR, o->Gx);
    hll(ny, o->SyL, o->SyR, o->GyL, o->GyR, o->HVyL, o->HVyR, o->Gy);
    boundary_condition(o);
}

/* ------------------------------------------------------------------------ */
/* SourceTerms (sources.F:56-548), CARTESIAN, no MANNING/METEO/VESSEL       */
/* ------------------------------------------------------------------------ */
static void wavemaker_mass(ofw_ctx *o) {
    const ofr TIME = o->TIME;
    if (o->p.wavemaker == 1) {
        /* WK_REG (sources.F:109-118) */
        ofr AA = tanh(PI_SP / (o->p.time_ramp * o->p.tperiod) * TIME) * o->D_gen;
        for (int J = o->jlo; J <= o->jhi; J++)
            for (int I = o->ilo; I <= o->ihi; I++) {
                ofr dxm = o->xmk_wk[I - 1] - o->p.xc_wk;
                C2(o->WaveMaker_Mass, I, J) =
                    AA * exp(-o->beta_gen * (dxm * dxm)) *
                    sin(o->rlamda * (o->ymk_wk[J - 1] - ZERO) - 2.0 * PI_SP / o->p.tperiod * TIME);
            }
    } else if (o->p.wavemaker == 2 && o->Cm) {
        /* JON_2D (sources.F:119-134) over the band */
        int nf = o->p.nfreq;
        ofr AA = tanh(PI_SP / (o->p.time_ramp / o->p.freq_peak) * TIME);
        ofr *BB = (ofr *)malloc(sizeof(ofr) * nf), *CC = (ofr *)malloc(sizeof(ofr) * nf);
        for (int k = 0; k < nf; k++) {
            BB[k] = cos(o->omgn_ir[k] * TIME);
            CC[k] = sin(o->omgn_ir[k] * TIME);
        }
        int bw = o->ihi - o->ilo + 1, bh = o->jhi - o->jlo + 1;
        for (int J = o->jlo; J <= o->jhi; J++)
            for (int I = o->ilo; I <= o->ihi; I++) {
                ofr s = ZERO;
                size_t b = (size_t)(I - o->ilo) + (size_t)(J - o->jlo) * bw;
                for (int k = 0; k < nf; k++)
                    s = s + AA * (o->Cm[b + (size_t)k * bw * bh] * BB[k] + o->Sm[b + (size_t)k * bw * bh] * CC[k]);
                C2(o->WaveMaker_Mass, I, J) = s;
            }
        free(BB);
        free(CC);
    }
}

void ofw_source_terms(ofw_ctx *o) {
    const int M = o->Mloc, N = o->Nloc;
    const ofr DX = o->p.DX, DY = o->p.DY, mdf = o->p.min_depth_frc;
    const ofr g1 = o->p.gamma1, g2 = o->p.gamma2;
    wavemaker_mass(o);
    /* nu_vis is default REAL (sources.F:69,190-224) */
    float *nu_vis = (float *)calloc((size_t)M * N, sizeof(float));
    if (o->p.viscosity_breaking) {
        for (size_t k = 0; k < (size_t)M * N; k++) nu_vis[k] = (float)o->nu_break[k];
    }
#define NV(I, J) nu_vis[(size_t)((I)-1) + (size_t)((J)-1) * (size_t)M]
    OMP_FOR
    for (int J = o->Jbeg; J <= o->Jend; J++)
        for (int I = o->Ibeg; I <= o->Iend; I++) {
            ofr U = C2(o->U, I, J), V = C2(o->V, I, J);
            ofr spd = sqrt(U * U + V * V);
            ofr m9 = (ofr)C2(o->MASK9, I, J);
            ofr FrcInsX = -C2(o->Cd, I, J) * U * spd;
            ofr SX = GRAV * (C2(o->Eta, I, J)) / DX * (X2(o->Depthx, I + 1, J) - X2(o->Depthx, I, J)) *
                            (ofr)C2(o->MASK, I, J) +
                        FrcInsX +
                        g1 * m9 * dmax(C2(o->H, I, J), mdf) *
                            (U * 0.5 * (C2(o->U4, I + 1, J) - C2(o->U4, I - 1, J)) / DX +
                             V * 0.5 * (C2(o->U4, I, J + 1) - C2(o->U4, I, J - 1)) / DY +
                             C2(o->U4, I, J) * 0.5 * (C2(o->U, I + 1, J) - C2(o->U, I - 1, J)) / DX +
                             C2(o->V4, I, J) * 0.5 * (C2(o->U, I, J + 1) - C2(o->U, I, J - 1)) / DY -
                             g2 * m9 * (C2(o->U1pp, I, J) + C2(o->U2, I, J) + C2(o->U3, I, J))) +
                        g1 * m9 * ((X2(o->P, I + 1, J) - X2(o->P, I, J)) / DX + (Y2(o->Q, I, J + 1) - Y2(o->Q, I, J)) / DY) *
                            (C2(o->U4, I, J) - C2(o->U1p, I, J)) +
                        C2(o->WaveMaker_Mass, I, J) * U;
            if (o->p.friction_sponge)
                SX = SX - C2(o->CD_4_SPONGE, I, J) * U * spd * C2(o->Depth, I, J);
            ofr FrcInsY = -C2(o->Cd, I, J) * V * spd;
            ofr SY = GRAV * (C2(o->Eta, I, J)) / DY * (Y2(o->Depthy, I, J + 1) - Y2(o->Depthy, I, J)) *
                            (ofr)C2(o->MASK, I, J) +
                        FrcInsY +
                        g1 * m9 * dmax(C2(o->H, I, J), mdf) *
                            (U * 0.5 * (C2(o->V4, I + 1, J) - C2(o->V4, I - 1, J)) / DX +
                             V * 0.5 * (C2(o->V4, I, J + 1) - C2(o->V4, I, J - 1)) / DY +
                             C2(o->U4, I, J) * 0.5 * (C2(o->V, I + 1, J) - C2(o->V, I - 1, J)) / DX +
                             C2(o->V4, I, J) * 0.5 * (C2(o->V, I, J + 1) - C2(o->V, I, J - 1)) / DY -
                             g2 * m9 * (C2(o->V1pp, I, J) + C2(o->V2, I, J) + C2(o->V3, I, J))) +
                        g1 * m9 * ((X2(o->P, I + 1, J) - X2(o->P, I, J)) / DX + (Y2(o->Q, I, J + 1) - Y2(o->Q, I, J)) / DY) *
                            (C2(o->V4, I, J) - C2(o->V1p, I, J)) +
                        C2(o->WaveMaker_Mass, I, J) * V;
            if (o->p.friction_sponge)
                SY = SY - C2(o->CD_4_SPONGE, I, J) * V * spd * C2(o->Depth, I, J);
            if (o->p.viscosity_breaking) {
                /* BreakSourceX/Y, non-PQ scheme (sources.F:428-456); the sums
                 * of two nu_vis values are float additions. */
                ofr nxp = (ofr)(float)(NV(I + 1, J) + NV(I, J));
                ofr nxm = (ofr)(float)(NV(I - 1, J) + NV(I, J));
                ofr nyp = (ofr)(float)(NV(I, J + 1) + NV(I, J));
                ofr nym = (ofr)(float)(NV(I, J - 1) + NV(I, J));
                ofr HUc = C2(o->HU, I, J), HVc = C2(o->HV, I, J);
                ofr BX = 0.5 / DX *
                                (nxp * 1.0 / DX * (C2(o->HU, I + 1, J) - HUc) -
                                 nxm * 1.0 / DX * (HUc - C2(o->HU, I - 1, J))) +
                            0.5 / DY *
                                (nyp * 1.0 / DY * (C2(o->HU, I, J + 1) - HUc) -
                                 nym * 1.0 / DY * (HUc - C2(o->HU, I, J - 1)));
                C2(o->BreakSourceX, I, J) = BX;
                SX = SX + BX;
                ofr BY = 0.5 / DX *
                                (nxp * 1.0 / DX * (C2(o->HV, I + 1, J) - HVc) -
                                 nxm * 1.0 / DX * (HVc - C2(o->HV, I - 1, J))) +
                            0.5 / DY *
                                (nyp * 1.0 / DY * (C2(o->HV, I, J + 1) - HVc) -
                                 nym * 1.0 / DY * (HVc - C2(o->HV, I, J - 1)));
                C2(o->BreakSourceY, I, J) = BY;
                SY = SY + BY;
            }
            C2(o->SourceX, I, J) = SX;
            C2(o->SourceY, I, J) = SY;
        }
#undef NV
    free(nu_vis);
}

/* ------------------------------------------------------------------------ */
/* tridiagonal solvers (tridiagnal.F:59-398), serial                        */
/* ------------------------------------------------------------------------ */
/* TRIDx_ser (tridiagnal.F:375-398) */
static void tridx_ser(ofw_ctx *o, ofr *A, ofr *C, ofr *D, ofr *Z) {
    OMP_FOR
    for (int JJ = o->Jbeg; JJ <= o->Jend; JJ++) {
        for (int II = o->Ibeg + 1; II <= o->Iend; II++) {
            ofr a = C2(A, II, JJ);
            if (a != ZERO) {
                C2(C, II, JJ) = C2(C, II, JJ) / a / (1.0 / a - C2(C, II - 1, JJ));
                C2(D, II, JJ) = (C2(D, II, JJ) / a - C2(D, II - 1, JJ)) / (1.0 / a - C2(C, II - 1, JJ));
            }
        }
        C2(Z, o->Iend, JJ) = C2(D, o->Iend, JJ);
        for (int II = o->Iend - 1; II >= o->Ibeg; II--)
            C2(Z, II, JJ) = C2(D, II, JJ) - C2(C, II, JJ) * C2(Z, II + 1, JJ);
    }
}

/* TRIDy_ser (tridiagnal.F:338-361) */
static void tridy_ser(ofw_ctx *o, ofr *A, ofr *C, ofr *D, ofr *Z) {
    OMP_FOR
    for (int II = o->Ibeg; II <= o->Iend; II++) {
        for (int JJ = o->Jbeg + 1; JJ <= o->Jend; JJ++) {
            ofr a = C2(A, II, JJ);
            if (a != ZERO) {
                C2(C, II, JJ) = C2(C, II, JJ) / a / (1.0 / a - C2(C, II, JJ - 1));
                C2(D, II, JJ) = (C2(D, II, JJ) / a - C2(D, II, JJ - 1)) / (1.0 / a - C2(C, II, JJ - 1));
            }
        }
        C2(Z, II, o->Jend) = C2(D, II, o->Jend);
        for (int JJ = o->Jend - 1; JJ >= o->Jbeg; JJ--)
            C2(Z, II, JJ) = C2(D, II, JJ) - C2(C, II, JJ) * C2(Z, II, JJ + 1);
    }
}

/* TRIDy_periodic (tridiagnal.F:59-325), serial branch */
static void tridy_periodic(ofw_ctx *o, ofr *a, ofr *c, ofr *d, ofr *f) {
    const int M = o->Mloc, N = o->Nloc, Jb = o->Jbeg, Je = o->Jend;
    const size_t nc = (size_t)M * N;
    ofr *c1 = (ofr *)malloc(nc * sizeof(ofr));
    ofr *y1 = (ofr *)calloc(nc, sizeof(ofr));
    ofr *y2 = (ofr *)calloc(nc, sizeof(ofr));
    ofr *a_beg = (ofr *)calloc((size_t)M + 1, sizeof(ofr));
    ofr *c_end = (ofr *)calloc((size_t)M + 1, sizeof(ofr));
    for (int I = o->Ibeg; I <= o->Iend; I++) {
        a_beg[I] = C2(a, I, Jb);
        c_end[I] = C2(c, I, Je);
    }
    for (int i = o->Ibeg; i <= o->Iend; i++) {
        C2(c, i, Jb) = C2(c, i, Jb) / (1 + c_end[i]);
        C2(d, i, Jb) = C2(d, i, Jb) / (1 + c_end[i]);
        C2(a, i, Je) = C2(a, i, Je) / (1 + a_beg[i]);
        C2(d, i, Je) = C2(d, i, Je) / (1 + a_beg[i]);
    }
    memcpy(c1, c, nc * sizeof(ofr));
    tridy_ser(o, a, c1, d, y1);
    for (int i = o->Ibeg; i <= o->Iend; i++) {
        C2(d, i, Jb) = 1.0 / (1.0 + c_end[i]);
        for (int j = Jb + 1; j <= Je - 1; j++) C2(d, i, j) = ZERO;
        C2(d, i, Je) = -1.0 / (1.0 + a_beg[i]);
    }
    tridy_ser(o, a, c, d, y2);
    for (int i = o->Ibeg; i <= o->Iend; i++) {
        ofr beta = (c_end[i] * C2(y1, i, Jb) - a_beg[i] * C2(y1, i, Je)) /
                      (1.0 - (c_end[i] * C2(y2, i, Jb) - a_beg[i] * C2(y2, i, Je)));
        for (int j = Jb; j <= Je; j++) C2(f, i, j) = C2(y1, i, j) + beta * C2(y2, i, j);
    }
    free(c1);
    free(y1);
    free(y2);
    free(a_beg);
    free(c_end);
}

/* ------------------------------------------------------------------------ */
/* ESTIMATE_HUV (etauv_solver.F:53-351) + GET_Eta_U_V_HU_HV (:365-604)      */
/* ------------------------------------------------------------------------ */
static void get_eta_u_v_hu_hv(ofw_ctx *o) {
    const int M = o->Mloc, N = o->Nloc;
    const size_t nc = (size_t)M * N;
    const ofr DX = o->p.DX, DY = o->p.DY, mdf = o->p.min_depth_frc;
    const ofr g1 = o->p.gamma1, g3 = o->p.gamma3, b1 = o->b1, b2 = o->b2;
    for (size_t k = 0; k < nc; k++) o->H[k] = o->Eta[k] * g3 + o->Depth[k];
    if (o->p.dispersion) {
        ofr *myA = (ofr *)calloc(nc, sizeof(ofr));
        ofr *myC = (ofr *)calloc(nc, sizeof(ofr));
        ofr *myD = (ofr *)calloc(nc, sizeof(ofr));
        ofr *myF = (ofr *)calloc(nc, sizeof(ofr));
        OMP_FOR
        for (int J = o->Jbeg; J <= o->Jend; J++)
            for (int I = o->Ibeg; I <= o->Iend; I++) {
                ofr dep = dmax(C2(o->Depth, I, J), mdf);
                ofr depl = dmax(C2(o->Depth, I - 1, J), mdf);
                ofr depr = dmax(C2(o->Depth, I + 1, J), mdf);
                ofr m9 = (ofr)C2(o->MASK9, I, J);
                ofr tmp1 = g1 * m9 * (b1 / 2.0 / DX / DX * dep * dep + b2 / DX / DX * depl * dep);
                ofr tmp2 = 1.0 + g1 * m9 * (-b1 / DX / DX * dep * dep - 2.0 * b2 / DX / DX * dep * dep);
                ofr tmp3 = g1 * m9 * (b1 / 2.0 / DX / DX * dep * dep + b2 / DX / DX * dep * depr);
                ofr tmp4 = C2(o->Ubar, I, J) * (ofr)C2(o->MASK, I, J) / dmax(C2(o->H, I, J), mdf) +
                              g1 * m9 * (-b1 / 2.0 * dep * dep * C2(o->Vxy, I, J) - b2 * dep * C2(o->DVxy, I, J));
                if (tmp2 != 0.0 || C2(o->MASK, I, J) > 0) {
                    C2(myA, I, J) = tmp1 / tmp2;
                    C2(myC, I, J) = tmp3 / tmp2;
                    C2(myD, I, J) = tmp4 / tmp2;
                } else {
                    C2(myA, I, J) = ZERO;
                    C2(myC, I, J) = ZERO;
                    C2(myD, I, J) = ZERO;
                }
            }
        tridx_ser(o, myA, myC, myD, myF);
        for (int J = o->Jbeg; J <= o->Jend; J++)
            for (int I = o->Ibeg; I <= o->Iend; I++) C2(o->U, I, J) = C2(myF, I, J);
        OMP_FOR
        for (int I = o->Ibeg; I <= o->Iend; I++)
            for (int J = o->Jbeg; J <= o->Jend; J++) {
                ofr dep = dmax(C2(o->Depth, I, J), mdf);
                ofr depl = dmax(C2(o->Depth, I, J - 1), mdf);
                ofr depr = dmax(C2(o->Depth, I, J + 1), mdf);
                ofr m9 = (ofr)C2(o->MASK9, I, J);
                ofr tmp1 = g1 * m9 * (b1 / 2.0 / DY / DY * dep * dep + b2 / DY / DY * depl * dep);
                ofr tmp2 = 1.0 + g1 * m9 * (-b1 / DY / DY * dep * dep - 2.0 * b2 / DY / DY * dep * dep);
                ofr tmp3 = g1 * m9 * (b1 / 2.0 / DY / DY * dep * dep + b2 / DY / DY * dep * depr);
                ofr tmp4 = C2(o->Vbar, I, J) * (ofr)C2(o->MASK, I, J) / dmax(C2(o->H, I, J), mdf) +
                              g1 * m9 * (-b1 / 2.0 * dep * dep * C2(o->Uxy, I, J) - b2 * dep * C2(o->DUxy, I, J));
                if (tmp2 != 0.0 || C2(o->MASK, I, J) > 0) {
                    C2(myA, I, J) = tmp1 / tmp2;
                    C2(myC, I, J) = tmp3 / tmp2;
                    C2(myD, I, J) = tmp4 / tmp2;
                } else {
                    C2(myA, I, J) = ZERO;
                    C2(myC, I, J) = ZERO;
                    C2(myD, I, J) = ZERO;
                }
            }
        if (o->p.periodic) tridy_periodic(o, myA, myC, myD, myF);
        else tridy_ser(o, myA, myC, myD, myF);
        for (int J = o->Jbeg; J <= o->Jend; J++)
            for (int I = o->Ibeg; I <= o->Iend; I++) C2(o->V, I, J) = C2(myF, I, J);
        free(myA);
        free(myC);
        free(myD);
        free(myF);
    } else {
        for (int J = o->Jbeg; J <= o->Jend; J++)
            for (int I = o->Ibeg; I <= o->Iend; I++) {
                C2(o->U, I, J) = C2(o->Ubar, I, J) / dmax(C2(o->H, I, J), mdf);
                C2(o->V, I, J) = C2(o->Vbar, I, J) / dmax(C2(o->H, I, J), mdf);
            }
    }
    const ofr fc = o->p.froude_cap;
    OMP_FOR
    for (int J = o->Jbeg; J <= o->Jend; J++)
        for (int I = o->Ibeg; I <= o->Iend; I++) {
            if (C2(o->MASK, I, J) < 1) {
                C2(o->Ubar, I, J) = ZERO;
                C2(o->Vbar, I, J) = ZERO;
                C2(o->U, I, J) = ZERO;
                C2(o->V, I, J) = ZERO;
                C2(o->HU, I, J) = ZERO;
                C2(o->HV, I, J) = ZERO;
            } else {
                ofr Hm = dmax(C2(o->H, I, J), mdf);
                ofr u = C2(o->U, I, J), v = C2(o->V, I, J);
                C2(o->HU, I, J) = Hm * u;
                C2(o->HV, I, J) = Hm * v;
                ofr Utotal = sqrt(u * u + v * v);
                ofr Fr = sqrt(GRAV * Hm);
                if (Utotal / Fr > fc) {
                    ofr Utheta = atan2(v, u);
                    C2(o->U, I, J) = fc * Fr * cos(Utheta);
                    C2(o->V, I, J) = fc * Fr * sin(Utheta);
                    C2(o->HU, I, J) = C2(o->U, I, J) * Hm;
                    C2(o->HV, I, J) = C2(o->V, I, J) * Hm;
                }
            }
        }
    if (!o->p.dispersion) {
        memcpy(o->Ubar, o->HU, nc * sizeof(ofr));
        memcpy(o->Vbar, o->HV, nc * sizeof(ofr));
    }
}

static const ofr RK_ALPHA[3] = {0.0, 3.0 / 4.0, 1.0 / 3.0};
static const ofr RK_BETA[3] = {1.0, 1.0 / 4.0, 2.0 / 3.0};

void ofw_estimate_huv(ofw_ctx *o, int istage) {
    const ofr DX = o->p.DX, DY = o->p.DY, DT = o->DT;
    const ofr al = RK_ALPHA[istage - 1], be = RK_BETA[istage - 1];
    const int wk = o->p.wavemaker;
    /* for radiation stress (etauv_solver.F:94-101), with the H of the
     * stage's start */
    OMP_FOR
    for (int J = o->Jbeg; J <= o->Jend; J++)
        for (int I = o->Ibeg; I <= o->Iend; I++) {
            const ofr pc = 0.5 * (X2(o->P, I + 1, J) + X2(o->P, I, J));
            const ofr qc = 0.5 * (Y2(o->Q, I, J + 1) + Y2(o->Q, I, J));
            const ofr hm = dmax(C2(o->H, I, J), o->p.min_depth_frc);
            C2(o->P_center, I, J) = pc;
            C2(o->Q_center, I, J) = qc;
            C2(o->U_davg, I, J) = pc / hm;
            C2(o->V_davg, I, J) = qc / hm;
        }
    OMP_FOR
    for (int J = o->Jbeg; J <= o->Jend; J++)
        for (int I = o->Ibeg; I <= o->Iend; I++) {
            ofr F_left = X2(o->P, I, J), F_right = X2(o->P, I + 1, J);
            ofr F_bottom = Y2(o->Q, I, J), F_top = Y2(o->Q, I, J + 1);
            ofr R1 = -1.0 / DX * (F_right * 1.0 + F_left * -1.0) - 1.0 / DY * (F_top * 1.0 + F_bottom * -1.0);
            if (wk == 1 || wk == 2) {
                ofr xmk = (I - o->Ibeg) * DX, ymk = (J - o->Jbeg) * DY;
                if (fabs(xmk - o->p.xc_wk) < o->Width_WK && fabs(ymk - o->p.yc_wk) < o->p.ywidth_wk / 2.0)
                    R1 = R1 + C2(o->WaveMaker_Mass, I, J);
            }
            C2(o->Wsurf, I, J) = R1; /* etauv_solver.F:247 */
            ofr eta = al * C2(o->Eta0, I, J) + be * (C2(o->Eta, I, J) + DT * R1);
            if (o->p.eta_limiter) {
                if (eta < o->p.trough_limit) eta = o->p.trough_limit;
                if (eta > o->p.crest_limit) eta = o->p.crest_limit;
            }
            C2(o->Eta, I, J) = eta;
        }
    OMP_FOR
    for (int J = o->Jbeg; J <= o->Jend; J++)
        for (int I = o->Ibeg; I <= o->Iend; I++) {
            ofr R2 = -1.0 / DX * (X2(o->Fx, I + 1, J) * 1.0 + X2(o->Fx, I, J) * -1.0) -
                        1.0 / DY * (Y2(o->Fy, I, J + 1) * 1.0 + Y2(o->Fy, I, J) * -1.0) + C2(o->SourceX, I, J);
            C2(o->Ubar, I, J) = al * C2(o->Ubar0, I, J) + be * (C2(o->Ubar, I, J) + DT * R2);
            ofr R3 = -1.0 / DX * (X2(o->Gx, I + 1, J) * 1.0 + X2(o->Gx, I, J) * -1.0) -
                        1.0 / DY * (Y2(o->Gy, I, J + 1) * 1.0 + Y2(o->Gy, I, J) * -1.0) + C2(o->SourceY, I, J);
            C2(o->Vbar, I, J) = al * C2(o->Vbar0, I, J) + be * (C2(o->Vbar, I, J) + DT * R3);
        }
    get_eta_u_v_hu_hv(o);
}

/* ------------------------------------------------------------------------ */
/* UPDATE_MASK (masks.F:51-205), no UseEtaScreen, no IGNORE_BIG_SLOPE      */
/* ------------------------------------------------------------------------ */
void ofw_update_mask(ofw_ctx *o) {
    const int M = o->Mloc, N = o->Nloc;
    const size_t nc = (size_t)M * N;
    int *MASKtmp = (int *)malloc(nc * sizeof(int));
    memcpy(MASKtmp, o->MASK, nc * sizeof(int));
    for (int J = o->Jbeg - 2; J <= o->Jend + 2; J++)
        for (int I = o->Ibeg - 2; I <= o->Iend + 2; I++) {
            if (C2(o->MASK_STRUC, I, J) == 1) {
                ofr eta = C2(o->Eta, I, J);
                if (C2(o->MASK, I, J) < 1) {
                    if (eta > -C2(o->Depth, I, J)) C2(MASKtmp, I, J) = 1;
                    if (C2(o->MASK, I - 1, J) == 1 && C2(o->Eta, I - 1, J) > eta) C2(MASKtmp, I, J) = 1;
                    if (C2(o->MASK, I + 1, J) == 1 && C2(o->Eta, I + 1, J) > eta) C2(MASKtmp, I, J) = 1;
                    if (C2(o->MASK, I, J - 1) == 1 && C2(o->Eta, I, J - 1) > eta) C2(MASKtmp, I, J) = 1;
                    if (C2(o->MASK, I, J + 1) == 1 && C2(o->Eta, I, J + 1) > eta) C2(MASKtmp, I, J) = 1;
                } else {
                    if (eta < -C2(o->Depth, I, J)) C2(MASKtmp, I, J) = 0;
                }
            }
            if (C2(o->MASK, I, J) < 1) {
                X2(o->Depthx, I, J) = C2(o->Depth, I - 1, J);
                X2(o->Depthx, I + 1, J) = C2(o->Depth, I + 1, J);
                Y2(o->Depthy, I, J) = C2(o->Depth, I, J - 1);
                Y2(o->Depthy, I, J + 1) = C2(o->Depth, I, J + 1);
            }
        }
    memcpy(o->MASK, MASKtmp, nc * sizeof(int));
    /* MASK9 = MASK9tmp: the ring outside Ibeg-1..Iend+1 x Jbeg-1..Jend+1 is
     * never written in the reference; it is 0 here. */
    int *MASK9tmp = (int *)calloc(nc, sizeof(int));
    for (int J = o->Jbeg - 1; J <= o->Jend + 1; J++)
        for (int I = o->Ibeg - 1; I <= o->Iend + 1; I++) {
            if (o->p.viscosity_breaking) {
                C2(MASK9tmp, I, J) = 1;
            } else {
                int m = C2(o->MASK, I, J) * C2(o->MASK, I - 1, J) * C2(o->MASK, I + 1, J) *
                        C2(o->MASK, I + 1, J + 1) * C2(o->MASK, I, J + 1) * C2(o->MASK, I - 1, J + 1) *
                        C2(o->MASK, I + 1, J - 1) * C2(o->MASK, I, J - 1) * C2(o->MASK, I - 1, J - 1);
                if (fabs(C2(o->Eta, I, J)) / dmax(C2(o->Depth, I, J), o->p.min_depth_frc) > o->p.swe_eta_dep)
                    m = 0;
                C2(MASK9tmp, I, J) = m;
            }
        }
    memcpy(o->MASK9, MASK9tmp, nc * sizeof(int));
    free(MASKtmp);
    free(MASK9tmp);
}

/* ------------------------------------------------------------------------ */
/* WAVE_BREAKING / BREAKING (breaker.F:60-353), default branch             */
/* ------------------------------------------------------------------------ */
void ofw_wave_breaking(ofw_ctx *o) {
    if (!o->p.show_breaking) return;
    const ofr DX = o->p.DX, DY = o->p.DY, DT = o->DT, mdf = o->p.min_depth_frc;
    const ofr Cbrk1 = o->p.cbrk1, Cbrk2 = o->p.cbrk2, T_brk = o->T_brk;
    ofr *AGE = o->AGE;
    for (int J = o->Jbeg - 1; J <= o->Jend + 1; J++)
        for (int I = o->Ibeg - 1; I <= o->Iend + 1; I++) {
            ofr Hc = C2(o->H, I, J);
            ofr tmp3 = sqrt(GRAV * dmax(mdf, Hc));
            ofr tmp1 = Cbrk1 * tmp3;
            ofr tmp2 = Cbrk2 * tmp3;
            ofr ex = C2(o->ETAx, I, J), ey = C2(o->ETAy, I, J), et = C2(o->ETAT, I, J);
            ofr ANGLE = atan2(-ey, -ex) * 180.0 / PI_SP;
            ofr tmp4 = dmax(sqrt(ex * ex + ey * ey), SMALL);
            ofr age = C2(AGE, I, J);
            if (et >= tmp1 && (age == ZERO || age > T_brk)) {
                C2(AGE, I, J) = DT;
            } else if (age > ZERO) {
                C2(AGE, I, J) = age + DT;
            } else {
                ofr Cc = dmin(fabs(et) / tmp4, sqrt(GRAV * fabs(Hc)));
                ofr propxy = sqrt(DX * DX + DY * DY) / dmax(Cc, SMALL);
                ofr propx = sqrt(DX * DX) / dmax(Cc, SMALL);
                ofr propy = sqrt(DY * DY) / dmax(Cc, SMALL);
                if (et >= tmp2) {
                    ofr AGE1, AGE2, AGE3;
                    if (ANGLE >= ZERO && ANGLE < 90.0) {
                        AGE1 = C2(AGE, I - 1, J);
                        AGE2 = C2(AGE, I - 1, J - 1);
                        AGE3 = C2(AGE, I, J - 1);
                        if ((AGE1 >= DT && AGE1 > propx) || (AGE2 >= DT && AGE2 > propxy) ||
                            (AGE3 >= DT && AGE3 > propy))
                            C2(AGE, I, J) = DT;
                    }
                    if (ANGLE >= 90.0 && ANGLE < 180.0) {
                        AGE1 = C2(AGE, I + 1, J);
                        AGE2 = C2(AGE, I + 1, J - 1);
                        AGE3 = C2(AGE, I, J - 1);
                        if ((AGE1 >= DT && AGE1 > propx) || (AGE2 >= DT && AGE2 > propxy) ||
                            (AGE3 >= DT && AGE3 > propy))
                            C2(AGE, I, J) = DT;
                    }
                    if (ANGLE >= -180.0 && ANGLE < -90.0) {
                        AGE1 = C2(AGE, I + 1, J);
                        AGE2 = C2(AGE, I + 1, J + 1);
                        AGE3 = C2(AGE, I, J + 1);
                        if ((AGE1 >= DT && AGE1 > propx) || (AGE2 >= DT && AGE2 > propxy) ||
                            (AGE3 >= DT && AGE3 > propy))
                            C2(AGE, I, J) = DT;
                    }
                    if (ANGLE >= -90.0 && ANGLE < 0.0) {
                        AGE1 = C2(AGE, I, J + 1);
                        AGE2 = C2(AGE, I - 1, J + 1);
                        AGE3 = C2(AGE, I - 1, J);
                        if ((AGE1 >= DT && AGE1 > propy) || (AGE2 >= DT && AGE2 > propxy) ||
                            (AGE3 >= DT && AGE3 > propx))
                            C2(AGE, I, J) = DT;
                    }
                }
            }
            ofr xmk = (I - o->Ibeg) * DX, ymk = (J - o->Jbeg) * DY;
            ofr a = C2(AGE, I, J);
            if (fabs(xmk - o->p.xc_wk) < o->Width_WK && fabs(ymk - o->p.yc_wk) < o->p.ywidth_wk / 2.0) {
                if (et > dmin(tmp2, o->p.wavemaker_cbrk * tmp3)) {
                    ofr cap1 = 1.0 * (dmax(C2(o->Depth, I, J), mdf) + C2(o->Eta, I, J));
                    C2(o->nu_break, I, J) = cap1 * o->p.wavemaker_cbrk * tmp3 + o->p.nu_bkg;
                } else {
                    C2(o->nu_break, I, J) = ZERO + o->p.nu_bkg;
                }
            } else {
                if (a > ZERO && a < T_brk && et > tmp2) {
                    ofr cap1 = 1.0 * (dmax(C2(o->Depth, I, J), mdf) + C2(o->Eta, I, J));
                    C2(o->nu_break, I, J) = cap1 * tmp2 + o->p.nu_bkg;
                    /* roller and undertow (breaker.F:316-339); 0.45 is a
                     * default-REAL literal, 0.1638 a _SP one */
                    ofr C1 = dmax(fabs(et) / tmp4, sqrt(GRAV * fabs(Hc)));
                    ofr R = fabs((ofr)0.45f * et / dmax(C1, SMALL));
                    R = dmin(R, (ofr)0.1638f);
                    ofr u = C2(o->U, I, J), v = C2(o->V, I, J);
                    ofr rf = fabs(C1 - sqrt(u * u + v * v)) * R * (C2(o->Eta, I, J) - C2(o->ETAmean, I, J));
                    C2(o->ROLLER_FLUX, I, J) = rf;
                    C2(o->UNDERTOW_U, I, J) = -rf * cos(ANGLE * PI_SP / 180.0);
                    C2(o->UNDERTOW_V, I, J) = -rf * sin(ANGLE * PI_SP / 180.0);
                } else {
                    C2(o->nu_break, I, J) = ZERO + o->p.nu_bkg;
                }
            }
        }
}

/* SPONGE_DAMPING (sponge.F:52-66) */
void ofw_sponge_damping(ofw_ctx *o) {
    const size_t nc = (size_t)o->Mloc * o->Nloc;
    OMP_FOR
    for (size_t k = 0; k < nc; k++) {
        if ((ofr)o->MASK[k] > ZERO) o->Eta[k] = o->Eta[k] / o->SPONGE[k];
        o->U[k] = o->U[k] / o->SPONGE[k];
        o->V[k] = o->V[k] / o->SPONGE[k];
    }
}

/* CHECK_BLOWUP (misc.F:394-433): 1 if max|Eta| (interior) > EtaBlowVal */
int ofw_check_blowup(ofw_ctx *o) {
    ofr mx = 0.0;
    int nan = 0;
    for (int J = o->Jbeg; J <= o->Jend; J++)
        for (int I = o->Ibeg; I <= o->Iend; I++) {
            ofr a = fabs(C2(o->Eta, I, J));
            if (a != a) nan = 1;
            if (a > mx) mx = a;
        }
    return (mx > o->EtaBlowVal || nan) ? 1 : 0;
}

/* MAX_MIN_PROPERTY (misc.F:307-383): running maxima/minima over wet cells
 * of every Mloc x Nloc cell, each behind its OUT_* switch.  OUT_Hmax is
 * always on here (the GPU library keeps it behind track_hmax). */
void ofw_max_min_property(ofw_ctx *o) {
    const size_t nc = (size_t)o->Mloc * o->Nloc;
    for (size_t k = 0; k < nc; k++) {
        if (o->MASK[k] <= 0) continue;
        const ofr eta = o->Eta[k], u = o->U[k], v = o->V[k];
        if (eta > o->HeightMax[k]) o->HeightMax[k] = eta;
        if (o->p.track_hmin && eta < o->HeightMin[k]) o->HeightMin[k] = eta;
        if (o->p.track_umax) {
            const ofr maxv = sqrt(u * u + v * v);
            if (maxv > o->VelocityMax[k]) o->VelocityMax[k] = maxv;
        }
        if (o->p.track_mfmax) {
            const ofr maxv = (u * u + v * v) * (o->H[k]);
            if (maxv > o->MomentumFluxMax[k]) o->MomentumFluxMax[k] = maxv;
        }
    }
}

/* the radiation-stress, momentum-flux and breaking-dissipation sums of one
 * cell (mixing.F:156-167 and 270-281), with the ETAmean and U_davg_mean the
 * caller's branch has at that point */
static void radiation_sums(ofw_ctx *o, size_t k, ofr DT) {
    const ofr ud = o->U_davg[k] - o->U_davg_mean[k], vd = o->V_davg[k] - o->V_davg_mean[k];
    const ofr hd = o->Eta[k] - o->ETAmean[k] + o->Depth[k];
    const ofr u = o->U[k], v = o->V[k];
    o->U_davg_sum[k] = o->U_davg[k] * DT + o->U_davg_sum[k];
    o->V_davg_sum[k] = o->V_davg[k] * DT + o->V_davg_sum[k];
    o->P_sum[k] = o->P_center[k] * DT + o->P_sum[k];
    o->Q_sum[k] = o->Q_center[k] * DT + o->Q_sum[k];
    o->UUsum[k] = ud * ud * hd * DT + o->UUsum[k];
    o->UVsum[k] = ud * vd * hd * DT + o->UVsum[k];
    o->VVsum[k] = vd * vd * hd * DT + o->VVsum[k];
    o->WWsum[k] = 0.25 * o->Wsurf[k] * o->Wsurf[k] * hd * DT + o->WWsum[k];
    o->FRCXsum[k] = u * sqrt(u * u + v * v) * DT + o->FRCXsum[k];
    o->FRCYsum[k] = v * sqrt(u * u + v * v) * DT + o->FRCYsum[k];
    o->BreakDissX_sum[k] = o->BreakDissX_sum[k] + o->BreakSourceX[k] * DT;
    o->BreakDissY_sum[k] = o->BreakDissY_sum[k] + o->BreakSourceY[k] * DT;
}

/* MIXING_STUFF / CALCULATE_MEAN (mixing.F:53-78, 108-305) from STEADY_TIME
 * on: time sums of Eta, U, V and (Eta-ETAmean)^2 over intervals of
 * T_INTV_mean, their means at the end of each interval, and zero-up-
 * crossing wave heights; the radiation-stress, momentum-flux and breaking-
 * dissipation sums and means, and at the end of an interval the gradient
 * fields DxSxx .. DxUVH on the interior (mixing.F:183-219).  Every sum and
 * mean starts at zero (the reference allocates some of them without setting
 * them).  The literals 4.004, 9.80 and 0.5*9.80 are default REAL. */
void ofw_mixing_stuff(ofw_ctx *o) {
    if (!(o->TIME >= o->p.steady_time)) return;
    const size_t nc = (size_t)o->Mloc * o->Nloc;
    const ofr DT = o->DT;
    o->T_sum = o->T_sum + DT;
    if (o->T_sum >= o->p.t_intv_mean) {
        const ofr Ts = o->T_sum;
        for (size_t k = 0; k < nc; k++) {
            const ofr d = o->Eta[k] - o->ETAmean[k];
            o->ETA2sum[k] = d * d * DT + o->ETA2sum[k];
            o->ETA2mean[k] = o->ETA2sum[k] / Ts;
            o->Usum[k] = o->U[k] * DT + o->Usum[k];
            o->Vsum[k] = o->V[k] * DT + o->Vsum[k];
            o->ETAsum[k] = o->Eta[k] * DT + o->ETAsum[k];
            o->Umean[k] = o->Usum[k] / Ts;
            o->Vmean[k] = o->Vsum[k] / Ts;
            o->ETAmean[k] = o->ETAsum[k] / Ts;
            radiation_sums(o, k, DT);
            o->U_davg_mean[k] = o->U_davg_sum[k] / Ts;
            o->V_davg_mean[k] = o->V_davg_sum[k] / Ts;
            o->P_mean[k] = o->P_sum[k] / Ts;
            o->Q_mean[k] = o->Q_sum[k] / Ts;
            o->UUmean[k] = o->UUsum[k] / Ts;
            o->UVmean[k] = o->UVsum[k] / Ts;
            o->VVmean[k] = o->VVsum[k] / Ts;
            o->WWmean[k] = o->WWsum[k] / Ts;
            o->FRCXmean[k] = o->FRCXsum[k] / Ts;
            o->FRCYmean[k] = o->FRCYsum[k] / Ts;
            o->BreakDissX[k] = o->BreakDissX_sum[k] / Ts;
            o->BreakDissY[k] = o->BreakDissY_sum[k] / Ts;
        }
        const ofr DX = o->p.DX, DY = o->p.DY, mdf = o->p.min_depth_frc;
        const ofr g98 = (ofr)9.80f, g49 = (ofr)(0.5f * 9.80f);
        for (int J = o->Jbeg; J <= o->Jend; J++)
            for (int I = o->Ibeg; I <= o->Iend; I++) {
#define RX(a) ((C2(o->a, I + 1, J) - C2(o->a, I - 1, J)) / 2.0 / DX)
#define RY(a) ((C2(o->a, I, J + 1) - C2(o->a, I, J - 1)) / 2.0 / DY)
#define HM(I_, J_) dmax(C2(o->Depth, I_, J_) + C2(o->ETAmean, I_, J_), mdf)
                C2(o->DxSxx, I, J) = RX(UUmean) - RX(WWmean) +
                                     g49 * (C2(o->ETA2mean, I + 1, J) - C2(o->ETA2mean, I - 1, J)) / 2.0 / DX;
                C2(o->DySxy, I, J) = RY(UVmean);
                C2(o->DySyy, I, J) = RY(VVmean) - RY(WWmean) +
                                     g49 * (C2(o->ETA2mean, I, J + 1) - C2(o->ETA2mean, I, J - 1)) / 2.0 / DY;
                C2(o->DxSxy, I, J) = RX(UVmean);
                C2(o->PgrdX, I, J) = g98 * (C2(o->Depth, I, J) + C2(o->ETAmean, I, J)) *
                                     (C2(o->ETAmean, I + 1, J) - C2(o->ETAmean, I - 1, J)) / 2.0 / DX;
                C2(o->PgrdY, I, J) = g98 * (C2(o->Depth, I, J) + C2(o->ETAmean, I, J)) *
                                     (C2(o->ETAmean, I, J + 1) - C2(o->ETAmean, I, J - 1)) / 2.0 / DY;
                C2(o->DxUUH, I, J) = (C2(o->P_mean, I + 1, J) * C2(o->P_mean, I + 1, J) / HM(I + 1, J) -
                                      C2(o->P_mean, I - 1, J) * C2(o->P_mean, I - 1, J) / HM(I - 1, J)) / 2.0 / DX;
                C2(o->DyUVH, I, J) = (C2(o->P_mean, I, J + 1) * C2(o->Q_mean, I, J + 1) / HM(I, J + 1) -
                                      C2(o->P_mean, I, J - 1) * C2(o->Q_mean, I, J - 1) / HM(I, J - 1)) / 2.0 / DY;
                C2(o->DyVVH, I, J) = (C2(o->Q_mean, I, J + 1) * C2(o->Q_mean, I, J + 1) / HM(I, J + 1) -
                                      C2(o->Q_mean, I, J - 1) * C2(o->Q_mean, I, J - 1) / HM(I, J - 1)) / 2.0 / DY;
                C2(o->DxUVH, I, J) = (C2(o->P_mean, I + 1, J) * C2(o->Q_mean, I + 1, J) / HM(I + 1, J) -
                                      C2(o->P_mean, I - 1, J) * C2(o->Q_mean, I - 1, J) / HM(I - 1, J)) / 2.0 / DX;
                C2(o->FRCXmean, I, J) = C2(o->FRCXmean, I, J) * C2(o->Cd, I, J);
                C2(o->FRCYmean, I, J) = C2(o->FRCYmean, I, J) * C2(o->Cd, I, J);
#undef RX
#undef RY
#undef HM
            }
        o->T_sum = o->T_sum - o->p.t_intv_mean;
        const ofr c4 = (ofr)(float)4.004;
        for (size_t k = 0; k < nc; k++) {
            o->Usum[k] = 0.0;
            o->Vsum[k] = 0.0;
            o->ETAsum[k] = 0.0;
            o->ETA2sum[k] = 0.0;
            o->U_davg_sum[k] = o->V_davg_sum[k] = o->P_sum[k] = o->Q_sum[k] = 0.0;
            o->UUsum[k] = o->UVsum[k] = o->VVsum[k] = o->WWsum[k] = 0.0;
            o->FRCXsum[k] = o->FRCYsum[k] = o->BreakDissX_sum[k] = o->BreakDissY_sum[k] = 0.0;
            o->SigWaveHeight[k] = c4 * sqrt(o->ETA2mean[k]);
            if (o->Num_Zero_Up[k] >= 2) {
                o->WaveHeightAve[k] = o->HavgSum[k] / o->Num_Zero_Up[k];
                o->WaveHeightRMS[k] = sqrt(o->HrmsSum[k] / o->Num_Zero_Up[k]);
            }
        }
    } else {
        for (size_t k = 0; k < nc; k++) {
            o->Usum[k] = o->U[k] * DT + o->Usum[k];
            o->Vsum[k] = o->V[k] * DT + o->Vsum[k];
            o->ETAsum[k] = o->Eta[k] * DT + o->ETAsum[k];
            const ofr d = o->Eta[k] - o->ETAmean[k];
            o->ETA2sum[k] = d * d * DT + o->ETA2sum[k];
            radiation_sums(o, k, DT);
            const ofr eta = o->Eta[k];
            if (eta > o->Emax[k]) o->Emax[k] = eta;
            if (eta < o->Emin[k]) o->Emin[k] = eta;
            const ofr tmpe = eta - o->ETAmean[k];
            const ofr tmp0 = o->Eta0[k] - o->ETAmean[k];
            if (tmpe > tmp0 && tmpe * tmp0 <= 0.0) {
                o->Num_Zero_Up[k] = o->Num_Zero_Up[k] + 1;
                if (o->Num_Zero_Up[k] >= 2) {
                    const ofr h = o->Emax[k] - o->Emin[k];
                    o->HavgSum[k] = (o->HavgSum[k] + o->Emax[k]) - o->Emin[k];  /* left to right */
                    o->HrmsSum[k] = o->HrmsSum[k] + h * h;
                }
                o->Emax[k] = -1000.0;
                o->Emin[k] = 1000.0;
            }
        }
    }
}

/* after the stages (main.F:496-517): MIXING_STUFF, MAX_MIN_PROPERTY,
 * CHECK_BLOWUP */
int ofw_end_step(ofw_ctx *o) {
    ofw_mixing_stuff(o);
    ofw_max_min_property(o);
    return ofw_check_blowup(o);
}

/* ------------------------------------------------------------------------ */
/* time loop body (main.F:284-535)                                          */
/* ------------------------------------------------------------------------ */
void ofw_begin_step(ofw_ctx *o) {
    const size_t nc = (size_t)o->Mloc * o->Nloc;
    memcpy(o->Eta0, o->Eta, nc * sizeof(ofr));
    memcpy(o->Ubar0, o->Ubar, nc * sizeof(ofr));
    memcpy(o->Vbar0, o->Vbar, nc * sizeof(ofr));
    ofw_exchange(o);
    ofw_estimate_dt(o);
    memcpy(o->U0, o->U, nc * sizeof(ofr));
    memcpy(o->V0, o->V, nc * sizeof(ofr));
}

void ofw_stage(ofw_ctx *o, int istage) {
    if (o->p.dispersion) ofw_cal_dispersion(o);
    ofw_fluxes(o);
    ofw_source_terms(o);
    ofw_estimate_huv(o, istage);
    ofw_update_mask(o);
    ofw_wave_breaking(o);
    ofw_exchange(o);
    if (o->p.direct_sponge) ofw_sponge_damping(o);
}

int ofw_step(ofw_ctx *o) {
    ofw_begin_step(o);
    for (int s = 1; s <= 3; s++) ofw_stage(o, s);
    return ofw_end_step(o);
}

/* ------------------------------------------------------------------------ */
/* INITIALIZATION (init.F:280-1272), the parts the hot path depends on      */
/* ------------------------------------------------------------------------ */

static void jon_spectrum(ofw_ctx *o);
static void jon_cm_sm(ofw_ctx *o);

/* integer power as gfortran's run-time helper: square-and-multiply */
static ofr powi(ofr x, int n) {
    ofr r = 1.0;
    int neg = n < 0;
    unsigned u = neg ? (unsigned)(-n) : (unsigned)n;
    while (u) {
        if (u & 1u) r *= x;
        x *= x;
        u >>= 1;
    }
    return neg ? 1.0 / r : r;
}

/* CALCULATE_SPONGE (sponge.F:591-767), serial */
static void calculate_sponge(ofw_ctx *o) {
    const int M = o->Mloc, N = o->Nloc;
    const ofr R = o->p.r_sponge, A = o->p.a_sponge;
    const size_t nc = (size_t)M * N;
    ofr *t1 = (ofr *)calloc(nc, sizeof(ofr));
    ofr *t2 = (ofr *)calloc(nc, sizeof(ofr));
    ofr *S = o->SPONGE;
    const ofr floor_ = pow(A, powi(R, 50));
    if (o->p.sponge_west > ZERO) {
        int Iw = (int)(o->p.sponge_west / o->p.DX) + NGHOST;
        for (int J = 1; J <= N; J++)
            for (int I = 1; I <= M; I++) {
                ofr lim = C2(S, I, J) > 1.0 ? C2(S, I, J) : 1.0;
                ofr ri = powi(R, 50 * (I - 1) / (Iw - 1));
                C2(t1, I, J) = dmax(pow(A, ri), lim);
            }
    }
    if (o->p.sponge_east > ZERO) {
        int Iw = (int)(o->p.sponge_east / o->p.DX) + NGHOST;
        for (int J = 1; J <= N; J++)
            for (int I = 1; I <= M; I++) {
                ofr lim = C2(S, I, J) > 1.0 ? C2(S, I, J) : 1.0;
                ofr ri = powi(R, 50 * (M - I) / (Iw - 1));
                C2(t2, I, J) = dmax(pow(A, ri), lim);
            }
    }
    for (size_t k = 0; k < nc; k++) {
        S[k] = t1[k] > t2[k] ? t1[k] : t2[k];
        if (S[k] < floor_) S[k] = 1.0;
    }
    if (o->p.sponge_south > ZERO) {
        int Iw = (int)(o->p.sponge_south / o->p.DY) + NGHOST;
        for (int I = 1; I <= M; I++)
            for (int J = 1; J <= N; J++) {
                ofr lim = C2(S, I, J) > 1.0 ? C2(S, I, J) : 1.0;
                ofr ri = powi(R, 50 * (J - 1) / (Iw - 1));
                C2(t1, I, J) = dmax(pow(A, ri), lim);
            }
    }
    if (o->p.sponge_north > ZERO) {
        int Iw = (int)(o->p.sponge_north / o->p.DY) + NGHOST;
        for (int I = 1; I <= M; I++)
            for (int J = 1; J <= N; J++) {
                ofr lim = C2(S, I, J) > 1.0 ? C2(S, I, J) : 1.0;
                ofr ri = powi(R, 50 * (N - J) / (Iw - 1));
                C2(t2, I, J) = dmax(pow(A, ri), lim);
            }
    }
    for (size_t k = 0; k < nc; k++) {
        S[k] = t1[k] > t2[k] ? t1[k] : t2[k];
        if (S[k] < floor_) S[k] = 1.0;
    }
    free(t1);
    free(t2);
}

/* WK_WAVEMAKER_REGULAR_WAVE (wavemaker.F:2369-2405); default-REAL literals
 * widened from float. */
static void wk_regular(ofw_ctx *o) {
    const ofr F1_3 = (ofr)(1.0f / 3.0f);
    double theta = o->p.theta_wk * PI_SP / 180.0;
    ofr alpha = (ofr)(float)-0.39;
    ofr alpha1 = alpha + F1_3;
    double omgn = 2.0 * PI_SP / o->p.tperiod;
    ofr h_gen = o->p.dep_wk;
    ofr tb = omgn * omgn * h_gen / GRAV;
    ofr tc = 1.0 + tb * alpha;
    ofr wkn = sqrt((tc - sqrt(tc * tc - 4.0 * alpha1 * tb)) / (2.0 * alpha1)) / h_gen;
    double C_phase = 1.0 / wkn / o->p.tperiod * 2.0 * PI_SP;
    ofr wave_length = C_phase * o->p.tperiod;
    o->rlamda = wkn * sin(theta);
    o->Width_WK = o->p.delta_wk * wave_length / 2.0;
    o->beta_gen = 80.0 / (o->p.delta_wk * o->p.delta_wk) / (wave_length * wave_length);
    ofr rl_gen = wkn * cos(theta);
    ofr rI = sqrt((ofr)(float)3.14159 / o->beta_gen) * exp(-(rl_gen * rl_gen) / 4.0 / o->beta_gen);
    ofr wh = wkn * h_gen;
    o->D_gen = 2.0 * o->p.amp_wk * cos(theta) *
               (omgn * omgn - alpha1 * GRAV * powi(wkn, 4) * powi(h_gen, 3)) /
               (omgn * wkn * rI * (1.0 - alpha * (wh * wh)));
}

int ofw_init(ofw_ctx *o) {
    const int M = o->Mloc, N = o->Nloc, M1 = o->Mloc1, N1 = o->Nloc1;
    const size_t nc = (size_t)M * N;
    const ofr mdf = o->p.min_depth_frc, g1 = o->p.gamma1, g3 = o->p.gamma3;
    /* dispersion coefficients (init.F:656-664) */
    ofr br = o->p.beta_ref;
    o->a1 = br * br / 2.0 - 1.0 / 6.0;
    o->a2 = br + 1.0 / 2.0;
    o->b1 = br * br;
    o->b2 = br;
    o->Beta_1 = br + 1.0;
    o->Beta_2 = (1.0 / 5.0) * (1.0 / 5.0) / 1.0;
    if (!o->p.dispersion) {
        o->p.gamma1 = ZERO;
        o->p.gamma2 = ZERO;
    }
    /* depth ghosts (init.F:789-794) */
    phi_coll(o, o->Depth, 1);
    /* face depths (init.F:811-829) */
    for (int J = 1; J <= N; J++)
        for (int I = 2; I <= M; I++) X2(o->Depthx, I, J) = 0.5 * (C2(o->Depth, I - 1, J) + C2(o->Depth, I, J));
    for (int J = 1; J <= N; J++) {
        X2(o->Depthx, 1, J) = 0.5 * (3.0 * C2(o->Depth, 1, J) - C2(o->Depth, 2, J));
        X2(o->Depthx, M1, J) = 0.5 * (3.0 * C2(o->Depth, M, J) - C2(o->Depth, M - 1, J));
    }
    for (int J = 2; J <= N; J++)
        for (int I = 1; I <= M; I++) Y2(o->Depthy, I, J) = 0.5 * (C2(o->Depth, I, J - 1) + C2(o->Depth, I, J));
    for (int I = 1; I <= M; I++) {
        Y2(o->Depthy, I, 1) = 0.5 * (3.0 * C2(o->Depth, I, 1) - C2(o->Depth, I, 2));
        Y2(o->Depthy, I, N1) = 0.5 * (3.0 * C2(o->Depth, I, N) - C2(o->Depth, I, N - 1));
    }
    /* EtaBlowVal (init.F:847) */
    ofr mx = 0.0;
    for (int J = o->Jbeg; J <= o->Jend; J++)
        for (int I = o->Ibeg; I <= o->Iend; I++) mx = dmax(mx, fabs(C2(o->Depth, I, J)));
    o->EtaBlowVal = 100.0 * mx;
    /* Cd (init.F:854-890), fixed value */
    for (size_t k = 0; k < nc; k++) o->Cd[k] = o->p.cd_fixed;
    /* wavemaker (init.F:963) */
    if (o->p.wavemaker == 1) wk_regular(o);
    if (o->p.wavemaker == 2) {
        if (!o->phi1) return -1;
        jon_spectrum(o);
    }
    /* sponges (init.F:966-989) */
    if (o->p.direct_sponge) calculate_sponge(o);
    /* MASK and dry Eta (init.F:1000-1014) */
    for (int J = 1; J <= N; J++)
        for (int I = 1; I <= M; I++) {
            if (C2(o->Eta, I, J) < -C2(o->Depth, I, J)) {
                C2(o->MASK, I, J) = 0;
                C2(o->Eta, I, J) = -o->p.min_depth - C2(o->Depth, I, J);
            } else {
                C2(o->MASK, I, J) = 1;
            }
        }
    /* H, HU, HV (init.F:1016-1018) */
    for (size_t k = 0; k < nc; k++) {
        o->H[k] = dmax(o->Eta[k] * g3 + o->Depth[k], mdf);
        o->HU[k] = o->H[k] * o->U[k];
        o->HV[k] = o->H[k] * o->V[k];
    }
    /* CAL_DISPERSION at initialisation (init.F:1021): MASK9 is still all 0
     * and DT is 0 */
    if (o->p.dispersion) ofw_cal_dispersion(o);
    for (size_t k = 0; k < nc; k++) {
        o->Ubar[k] = o->HU[k] + o->p.gamma1 * o->U1p[k] * o->H[k];
        o->Vbar[k] = o->HV[k] + o->p.gamma1 * o->V1p[k] * o->H[k];
    }
    /* structures (init.F:1106-1116) */
    for (size_t k = 0; k < nc; k++) {
        if (o->MASK_STRUC[k] == 0) o->Depth[k] = -LARGE;
        o->MASK[k] = o->MASK[k] * o->MASK_STRUC[k];
    }
    /* MASK9 interior (init.F:1153-1159) */
    for (int J = o->Jbeg; J <= o->Jend; J++)
        for (int I = o->Ibeg; I <= o->Iend; I++)
            C2(o->MASK9, I, J) = C2(o->MASK, I, J) * C2(o->MASK, I - 1, J) * C2(o->MASK, I + 1, J) *
                                 C2(o->MASK, I + 1, J + 1) * C2(o->MASK, I, J + 1) * C2(o->MASK, I - 1, J + 1) *
                                 C2(o->MASK, I + 1, J - 1) * C2(o->MASK, I, J - 1) * C2(o->MASK, I - 1, J - 1);
    /* dry face depths (init.F:1210-1219) */
    for (int J = 2; J <= N - 1; J++)
        for (int I = 2; I <= M - 1; I++)
            if (C2(o->MASK, I, J) < 1) {
                X2(o->Depthx, I, J) = C2(o->Depth, I - 1, J);
                X2(o->Depthx, I + 1, J) = C2(o->Depth, I + 1, J);
                Y2(o->Depthy, I, J) = C2(o->Depth, I, J - 1);
                Y2(o->Depthy, I, J + 1) = C2(o->Depth, I, J + 1);
            }
    if (o->p.show_breaking) o->T_brk = 20.0;
    /* wavemaker band (init.F:1236-1268) */
    o->ilo = o->Iend + 1;
    o->ihi = o->Ibeg - 1;
    o->jlo = o->Jend + 1;
    o->jhi = o->Jbeg - 1;
    for (int J = o->Jbeg; J <= o->Jend; J++) {
        o->ymk_wk[J - 1] = (J - o->Jbeg) * o->p.DY;
        if (fabs(o->ymk_wk[J - 1] - o->p.yc_wk) < o->p.ywidth_wk / 2.0) {
            if (J < o->jlo) o->jlo = J;
            if (J > o->jhi) o->jhi = J;
        }
    }
    for (int I = o->Ibeg; I <= o->Iend; I++) {
        o->xmk_wk[I - 1] = (I - o->Ibeg) * o->p.DX;
        if (fabs(o->xmk_wk[I - 1] - o->p.xc_wk) < o->Width_WK) {
            if (I < o->ilo) o->ilo = I;
            if (I > o->ihi) o->ihi = I;
        }
    }
    if (o->p.wavemaker == 2) jon_cm_sm(o);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* JON_2D: WK_EQUAL_DFREQ_IRREGULAR_WAVE (wavemaker.F:2128-2357) and        */
/* CALCULATE_Cm_Sm (wavemaker.F:831-891) on the band only                  */
/* ------------------------------------------------------------------------ */
void ofw_set_phases(ofw_ctx *o, const double *phi1) {
    size_t n = (size_t)o->p.nfreq * o->p.ntheta;
    free(o->phi1);
    o->phi1 = (double *)malloc(sizeof(double) * (n ? n : 1));
    memcpy(o->phi1, phi1, sizeof(double) * n);
}

/* theta of direction ktheta (1-based), clamped to +-pi/2 (wavemaker.F:2211-2216) */
static ofr jon_theta(const ofw_params *p, int ktheta) {
    double theta = -PI_SP / 3.0 + p->theta_peak * PI_SP / 180.0 +
                   2.0 / 3.0 * PI_SP / ((double)(float)p->ntheta - 1.0) * ((double)(float)ktheta - 1.0);
    if (theta > 0.5 * PI_SP) theta = 0.5 * PI_SP;
    if (theta < -0.5 * PI_SP) theta = -0.5 * PI_SP;
    return theta;
}

static void jon_spectrum(ofw_ctx *o) {
    const ofw_params *p = &o->p;
    const int mf = p->nfreq, mt = p->ntheta;
    const ofr h_gen = p->dep_wk, fm = p->freq_peak, delta = p->delta_wk;
    ofr *freq = (ofr *)calloc((size_t)mf, sizeof(ofr));
    ofr *EB = (ofr *)calloc((size_t)mf, sizeof(ofr));
    ofr *AG = (ofr *)calloc((size_t)mt, sizeof(ofr));
    free(o->omgn_ir);
    free(o->jon_dgen);
    free(o->jon_rlamda);
    free(o->jon_betagen);
    o->omgn_ir = (double *)calloc((size_t)mf, sizeof(double));
    o->jon_dgen = (double *)calloc((size_t)mf * mt, sizeof(double));
    o->jon_rlamda = (double *)calloc((size_t)mf * mt, sizeof(double));
    o->jon_betagen = (double *)calloc((size_t)mf, sizeof(double));
    ofr df = (p->freq_max - p->freq_min) / (mf - 1.0);
    ofr Ef = ZERO;
    for (int kff = 1; kff <= mf; kff++) {
        ofr f = p->freq_min + (kff - 1) * df;
        freq[kff - 1] = f;
        /* JON spectra use phi = 1 (wavemaker.F:2164-2166) */
        ofr phi = 1.0;
        ofr sigma_spec = 0.07;
        if (f > fm) sigma_spec = 0.09;
        ofr r = f / fm - 1.0;
        double Etma = GRAV * GRAV * powi(f, -5) * powi(2.0 * PI_SP, -4) * phi *
                      exp(-5.0 / 4.0 * powi(f / fm, -4)) *
                      pow(p->gamma_tma, exp(-(r * r) / (2.0 * (sigma_spec * sigma_spec))));
        EB[kff - 1] = Etma * df;
        Ef = Ef + EB[kff - 1];
    }
    if (mt == 1) {
        AG[0] = 1.0;
    } else if (p->spreading == 1) {
        /* cos^2s((theta - theta_p)/2), normalised to unit sum like the
         * reference's AG (an extension: the reference has no cos^2s) */
        ofr sumAG = 0.0;
        for (int kt = 1; kt <= mt; kt++) {
            ofr th = jon_theta(p, kt);
            double c = cos((th - p->theta_peak * PI_SP / 180.0) / 2.0);
            AG[kt - 1] = pow(fabs(c), 2.0 * p->spread_s);
            sumAG = sumAG + AG[kt - 1];
        }
        for (int kt = 0; kt < mt; kt++) AG[kt] = fabs(AG[kt] / sumAG);
    } else {
        double sigma_theta = p->sigma_theta * PI_SP / 180.0;
        int N_spec = (int)(20.0 / sigma_theta);
        ofr sumAG = 0.0;
        for (int kt = 1; kt <= mt; kt++) {
            ofr th = jon_theta(p, kt);
            double ag = 1.0 / (2.0 * PI_SP);
            for (int k_n = 1; k_n <= N_spec; k_n++) {
                ofr a = (ofr)(float)k_n * sigma_theta;
                ag = ag + (1.0 / PI_SP) * exp(-0.5 * (a * a)) * cos(k_n * (th - p->theta_peak * PI_SP / 180.0));
            }
            AG[kt - 1] = ag;
            sumAG = sumAG + ag;
        }
        for (int kt = 0; kt < mt; kt++) AG[kt] = fabs(AG[kt] / sumAG);
    }
    ofr alpha_spec = p->hmo * p->hmo / 16.0 / Ef;
    const ofr alpha = -0.39, alpha1 = alpha + 1.0 / 3.0;
    ofr wave_length = 0.0;
    for (int kf = 1; kf <= mf; kf++)
        for (int kt = 1; kt <= mt; kt++) {
            ofr Hmo_each = 4.0 * sqrt((alpha_spec * EB[kf - 1] * AG[kt - 1]));
            ofr ap = Hmo_each / sqrt(2.0) / 2.0;
            double theta = (mt == 1) ? p->theta_peak * PI_SP / 180.0 : jon_theta(p, kt);
            double omgn = 2.0 * PI_SP * freq[kf - 1];
            o->omgn_ir[kf - 1] = omgn;
            ofr tb = omgn * omgn * h_gen / GRAV;
            ofr tc = 1.0 + tb * alpha;
            ofr wkn = sqrt((tc - sqrt(tc * tc - 4.0 * alpha1 * tb)) / (2.0 * alpha1)) / h_gen;
            ofr C_phase;
            if (wkn == 0.0) {
                wkn = SMALL;
                C_phase = sqrt(GRAV * h_gen);
                wave_length = C_phase / fm;
            } else {
                C_phase = 1.0 / wkn * fm * 2.0 * PI_SP;
                wave_length = C_phase / fm;
            }
            if (p->periodic) {
                /* snap the direction to a y-periodic wavenumber
                 * (wavemaker.F:2262-2296) */
                ofr tmp1 = wkn, tmp2 = 0.0, tmp3 = ZERO;
                int I = 0;
                if (theta > ZERO) {
                    while (tmp3 < theta) {
                        I = I + 1;
                        tmp2 = I * 2.0 * PI_SP / p->DY / (p->Nglob - 1.0);
                        if (tmp2 >= tmp1) tmp3 = PI_SP / 2.0;
                        else tmp3 = asin(tmp2 / tmp1);
                    }
                    if (tmp2 < tmp1) tmp3 = asin((I - 1) * 2.0 * PI_SP / p->DY / (p->Nglob - 1.0) / tmp1);
                    theta = tmp3;
                } else if (theta < ZERO) {
                    while (tmp3 > theta) {
                        I = I + 1;
                        tmp2 = I * 2.0 * PI_SP / p->DY / (p->Nglob - 1.0);
                        if (tmp2 >= tmp1) tmp3 = -PI_SP / 2.0;
                        else tmp3 = -asin(tmp2 / tmp1);
                    }
                    if (tmp2 < tmp1) tmp3 = -asin((I - 1) * 2.0 * PI_SP / p->DY / (p->Nglob - 1.0) / tmp1);
                    theta = tmp3;
                } else {
                    theta = tmp3;
                }
            }
            size_t k2 = (size_t)(kf - 1) + (size_t)(kt - 1) * mf;
            o->jon_rlamda[k2] = wkn * sin(theta);
            ofr bg = 80.0 / (delta * delta) / (wave_length * wave_length);
            o->jon_betagen[kf - 1] = bg;
            ofr rl_gen = wkn * cos(theta);
            double rI = sqrt(PI_SP / bg) * exp(-(rl_gen * rl_gen) / 4.0 / bg);
            ofr wh = wkn * h_gen;
            o->jon_dgen[k2] = 2.0 * ap * cos(theta) *
                              (omgn * omgn - alpha1 * GRAV * powi(wkn, 4) * powi(h_gen, 3)) /
                              (omgn * wkn * rI * (1.0 - alpha * (wh * wh)));
        }
    o->Width_WK = delta * wave_length / 2.0;
    free(freq);
    free(EB);
    free(AG);
}

/* CALCULATE_Cm_Sm (wavemaker.F:831-891) restricted to the band */
static void jon_cm_sm(ofw_ctx *o) {
    const int mf = o->p.nfreq, mt = o->p.ntheta;
    int bw = o->ihi - o->ilo + 1, bh = o->jhi - o->jlo + 1;
    free(o->Cm);
    free(o->Sm);
    o->Cm = o->Sm = NULL;
    if (bw <= 0 || bh <= 0) return;
    size_t n = (size_t)bw * bh * mf;
    o->Cm = (double *)calloc(n, sizeof(double));
    o->Sm = (double *)calloc(n, sizeof(double));
    for (int J = o->jlo; J <= o->jhi; J++)
        for (int I = o->ilo; I <= o->ihi; I++) {
            size_t b = (size_t)(I - o->ilo) + (size_t)(J - o->jlo) * bw;
            for (int kf = 1; kf <= mf; kf++) {
                ofr cm = ZERO, sm = ZERO;
                for (int kt = 1; kt <= mt; kt++) {
                    size_t k2 = (size_t)(kf - 1) + (size_t)(kt - 1) * mf;
                    ofr dxm = (I - o->Ibeg) * o->p.DX - o->p.xc_wk;
                    ofr amp = o->jon_dgen[k2] * exp(-o->jon_betagen[kf - 1] * (dxm * dxm));
                    ofr arg = o->jon_rlamda[k2] * ((J - o->Jbeg) * o->p.DY - ZERO) + o->phi1[k2];
                    cm = cm + amp * cos(arg);
                    sm = sm + amp * sin(arg);
                }
                o->Cm[b + (size_t)(kf - 1) * bw * bh] = cm;
                o->Sm[b + (size_t)(kf - 1) * bw * bh] = sm;
            }
        }
}

const double *ofw_jon_omega(ofw_ctx *o) { return o->omgn_ir; }
const double *ofw_jon_cm(ofw_ctx *o) { return o->Cm; }
const double *ofw_jon_sm(ofw_ctx *o) { return o->Sm; }
const double *ofw_jon_dgen(ofw_ctx *o) { return o->jon_dgen; }
const double *ofw_jon_rlamda(ofw_ctx *o) { return o->jon_rlamda; }
const double *ofw_jon_betagen(ofw_ctx *o) { return o->jon_betagen; }
