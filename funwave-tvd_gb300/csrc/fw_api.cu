// fw_api.cu -- the C ABI of include/funwave_gpu.h: context creation, one
// device arena for all state, Fortran-layout field transfer, the stepping
// entry points and the CUDA-graph replay of whole steps.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <map>
#include <mutex>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "fw_init.h"
#include "fw_internal.h"

using namespace fw;

namespace {

const char *kErrText[] = {"ok",
                          "CUDA runtime error",
                          "device allocation failed",
                          "invalid argument",
                          "blow-up: max|eta| exceeds EtaBlowVal",
                          "non-finite eta",
                          "option not supported by this build",
                          "call out of order (context not initialised)",
                          "no usable CUDA device",
                          "checkpoint file unreadable, unwritable or malformed",
                          "a bounded device wait ran out"};

int cuda_status(fw_ctx *c, cudaError_t e) {
    if (e == cudaSuccess && c && c->sticky_error == 0) return FW_OK;
    if (c && !c->sticky_error && e != cudaSuccess) c->sticky_error = (int)e;
    return FW_ERR_CUDA;
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// field table: name -> device pointer, element kind and layout
enum Kind { CELL = 0, XFACE = 1, YFACE = 2 };
struct FieldRef {
    void *ptr;
    int kind;
    int is_mask;  // uint8 on the device, int32 on the host
};

template <typename T> bool find_field(fw_ctx *c, const char *name, FieldRef &r) {
    Fields<T> &f = c->F<T>();
    struct E {
        const char *n;
        void *p;
        int k;
        int m;
    } tab[] = {
        {"Eta", f.Eta, CELL, 0}, {"U", f.U, CELL, 0}, {"V", f.V, CELL, 0}, {"Ubar", f.Ubar, CELL, 0},
        {"Vbar", f.Vbar, CELL, 0}, {"HU", f.HU, CELL, 0}, {"HV", f.HV, CELL, 0}, {"H", f.H, CELL, 0},
        {"Eta0", f.Eta0, CELL, 0}, {"Ubar0", f.Ubar0, CELL, 0}, {"Vbar0", f.Vbar0, CELL, 0}, {"U0", f.U0, CELL, 0},
        {"V0", f.V0, CELL, 0}, {"Depth", f.Depth, CELL, 0}, {"Cd", f.Cd, CELL, 0}, {"SPONGE", f.SPONGE, CELL, 0},
        {"CD_4_SPONGE", f.CD4, CELL, 0}, {"U4", f.U4, CELL, 0}, {"V4", f.V4, CELL, 0}, {"U1p", f.U1p, CELL, 0},
        {"V1p", f.V1p, CELL, 0}, {"Udisp", f.Udisp, CELL, 0}, {"Vdisp", f.Vdisp, CELL, 0},
        {"ETAx", f.ETAx, CELL, 0}, {"ETAy", f.ETAy, CELL, 0}, {"ETAT", f.ETAT, CELL, 0}, {"AGE", f.AGE, CELL, 0},
        {"nu_break", f.nu, CELL, 0}, {"SourceX", f.SourceX, CELL, 0}, {"SourceY", f.SourceY, CELL, 0},
        {"WaveMaker_Mass", f.WM, CELL, 0}, {"HeightMax", f.Hmax, CELL, 0}, {"Depthx", f.Depthx, XFACE, 0},
        {"P", f.P, XFACE, 0}, {"Fx", f.Fx, XFACE, 0}, {"Gx", f.Gx, XFACE, 0}, {"Depthy", f.Depthy, YFACE, 0},
        {"Q", f.Q, YFACE, 0}, {"Fy", f.Fy, YFACE, 0}, {"Gy", f.Gy, YFACE, 0}, {"MASK", f.MASK, CELL, 1},
        {"MASK9", f.MASK9, CELL, 1}, {"MASK_STRUC", f.MASK_STRUC, CELL, 1},
        {"HeightMin", f.Hmin, CELL, 0}, {"VelocityMax", f.Umax, CELL, 0}, {"MomentumFluxMax", f.MFmax, CELL, 0},
        {"ROLLER_FLUX", f.ROLLER, CELL, 0}, {"UNDERTOW_U", f.UNDERTOW_U, CELL, 0}, {"UNDERTOW_V", f.UNDERTOW_V, CELL, 0},
        {"ETAmean", f.ETAmean, CELL, 0}, {"Umean", f.Umean, CELL, 0}, {"Vmean", f.Vmean, CELL, 0},
        {"ETA2mean", f.ETA2mean, CELL, 0}, {"SigWaveHeight", f.SigWH, CELL, 0},
        {"WaveHeightAve", f.WHave, CELL, 0}, {"WaveHeightRMS", f.WHrms, CELL, 0}, {"Emax", f.Emax, CELL, 0},
        {"Emin", f.Emin, CELL, 0}, {"Num_Zero_Up", f.NZU, CELL, 0},
    };
    for (auto &e : tab)
        if (std::strcmp(e.n, name) == 0) {
            if (!e.p) return false;  // a statistic that is switched off
            r.ptr = e.p;
            r.kind = e.k;
            r.is_mask = e.m;
            return true;
        }
    // CALCULATE_MEAN's radiation-stress planes (fw::RadPlane order), with
    // the reference's names
    static const char *const rad_names[fw::RP_KAHAN] = {
        "P_center", "Q_center", "U_davg", "V_davg", "Wsurf", "BreakSourceX", "BreakSourceY",
        "U_davg_sum", "V_davg_sum", "P_sum", "Q_sum", "UUsum", "UVsum", "VVsum", "WWsum", "FRCXsum", "FRCYsum",
        "BreakDissX_sum", "BreakDissY_sum",
        "U_davg_mean", "V_davg_mean", "P_mean", "Q_mean", "UUmean", "UVmean", "VVmean", "WWmean", "FRCXmean",
        "FRCYmean", "BreakDissX", "BreakDissY",
        "DxSxx", "DySxy", "DySyy", "DxSxy", "PgrdX", "PgrdY", "DxUUH", "DyUVH", "DyVVH", "DxUVH"};
    for (int k = 0; k < fw::RP_KAHAN; k++)
        if (std::strcmp(rad_names[k], name) == 0) {
            if (!f.rad) return false;
            r.ptr = f.rad + (size_t)k * (size_t)c->g.pitch * (size_t)(c->g.Nloc + 1);
            r.kind = CELL;
            r.is_mask = 0;
            return true;
        }
    return false;
}

void extent(const fw_ctx *c, int kind, int &w, int &h) {
    w = c->g.Mloc + (kind == XFACE ? 1 : 0);
    h = c->g.Nloc + (kind == YFACE ? 1 : 0);
}

// host (Fortran, double/int32, w x h) <-> device (pitched, T/uint8).
// double fields of the FP64 build move with one 2-D copy; float fields and
// masks go through a device staging plane and a conversion kernel.
template <typename T> int put_field(fw_ctx *c, const FieldRef &r, const void *host) {
    int w, h;
    extent(c, r.kind, w, h);
    cudaError_t e;
    if (!r.is_mask && sizeof(T) == sizeof(double)) {
        e = cudaMemcpy2DAsync(r.ptr, (size_t)c->g.pitch * sizeof(T), host, (size_t)w * sizeof(double),
                              (size_t)w * sizeof(double), (size_t)h, cudaMemcpyHostToDevice, c->stream);
    } else {
        const size_t esz = r.is_mask ? sizeof(int) : sizeof(double);
        e = cudaMemcpyAsync(c->staging, host, (size_t)w * h * esz, cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess) convert_in(c, c->staging, r.is_mask, r.ptr, w, h);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    return cuda_status(c, e);
}

template <typename T> int get_field(fw_ctx *c, const FieldRef &r, void *host) {
    int w, h;
    extent(c, r.kind, w, h);
    cudaError_t e;
    if (!r.is_mask && sizeof(T) == sizeof(double)) {
        e = cudaMemcpy2DAsync(host, (size_t)w * sizeof(double), r.ptr, (size_t)c->g.pitch * sizeof(T),
                              (size_t)w * sizeof(double), (size_t)h, cudaMemcpyDeviceToHost, c->stream);
    } else {
        const size_t esz = r.is_mask ? sizeof(int) : sizeof(double);
        convert_out(c, r.ptr, r.is_mask, c->staging, w, h);
        e = cudaMemcpyAsync(host, c->staging, (size_t)w * h * esz, cudaMemcpyDeviceToHost, c->stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    return cuda_status(c, e);
}

int put_named(fw_ctx *c, const char *name, const void *host) {
    FieldRef r;
    if (c->p.precision == FW_PREC_FP64) {
        if (!find_field<double>(c, name, r)) return FW_ERR_BAD_PARAM;
        return put_field<double>(c, r, host);
    }
    if (!find_field<float>(c, name, r)) return FW_ERR_BAD_PARAM;
    int rc = put_field<float>(c, r, host);
    if (rc == FW_OK && std::strcmp(name, "Depth") == 0) {
        // the double copy of the total-depth tests (UPDATE_MASK)
        FieldRef rd{c->ff.DepthD, 0, 0};
        rc = put_field<double>(c, rd, host);
    }
    return rc;
}

void fill_float_constants(Grid &g) {
    g.f_DX = (float)g.DX;
    g.f_DY = (float)g.DY;
    g.f_rdx = (float)g.rdx;
    g.f_rdy = (float)g.rdy;
    g.f_hdx = (float)(0.5 * g.rdx);
    g.f_hdy = (float)(0.5 * g.rdy);
    g.f_rdx2 = (float)(g.rdx * g.rdx);
    g.f_rdy2 = (float)(g.rdy * g.rdy);
    g.f_rdxy4 = (float)(0.25 * g.rdx * g.rdy);
    g.f_cx = (float)(0.5 * g.rdx * g.rdx);
    g.f_cy = (float)(0.5 * g.rdy * g.rdy);
    g.f_min_depth_frc = (float)g.min_depth_frc;
    g.f_gamma1 = (float)g.gamma1;
    g.f_gamma2 = (float)g.gamma2;
    g.f_gamma3 = (float)g.gamma3;
    g.f_Beta_1 = (float)g.Beta_1;
    g.f_Beta_2 = (float)g.Beta_2;
    g.f_b1 = (float)g.b1;
    g.f_b2 = (float)g.b2;
    g.f_hb1 = (float)(-0.5 * g.b1);
    g.f_cbrk1 = (float)g.cbrk1;
    g.f_cbrk2 = (float)g.cbrk2;
    g.f_wavemaker_cbrk = (float)g.wavemaker_cbrk;
    g.f_nu_bkg = (float)g.nu_bkg;
    g.f_T_brk = (float)g.T_brk;
    g.f_froude_cap = (float)g.froude_cap;
    g.f_swe_eta_dep = (float)g.swe_eta_dep;
    g.f_xc_wk = (float)g.xc_wk;
    g.f_yc_wk = (float)g.yc_wk;
    g.f_ywidth_wk = (float)g.ywidth_wk;
    g.f_width_wk = (float)g.width_wk;
    g.f_D_gen = (float)g.D_gen;
    g.f_beta_gen = (float)g.beta_gen;
    g.f_rlamda = (float)g.rlamda;
    g.f_trough = (float)g.trough;
    g.f_crest = (float)g.crest;
}

LinePart make_part(int L, int nlines) {
    LinePart lp;
    lp.L = L;
    lp.nlines = nlines;
    lp.red0 = 0;
    // chunks of at least 16 rows and at most 256 chunks per line (the
    // reduced system of 2P rows is solved by one block)
    lp.m = std::max(16, (L + 255) / 256);
    if (L < 2 * lp.m) {
        lp.m = L;
        lp.P = 1;
    } else {
        lp.P = L / lp.m;
    }
    lp.lgm = -1;
    for (int b = 0; b < 31; b++)
        if ((1 << b) == lp.m) lp.lgm = b;
    return lp;
}

// carve the arena: T fields, masks, double scratch, small tables
template <typename T> size_t carve(fw_ctx *c, char *base, bool assign) {
    const Grid &g = c->g;
    const size_t plane = (size_t)g.pitch * (size_t)(g.Nloc + 1);
    size_t off = 0;
    auto take = [&](size_t bytes) {
        size_t o = off;
        off = align256(off + bytes);
        return base + o;
    };
    Fields<T> f{};
    T **tf[] = {&f.Eta,   &f.U,     &f.V,     &f.Ubar,   &f.Vbar,  &f.HU,   &f.HV,    &f.H,     &f.Eta0,
                &f.Ubar0, &f.Vbar0, &f.U0,    &f.V0,     &f.Depth, &f.Depthx, &f.Depthy, &f.Cd, &f.SPONGE,
                &f.CD4,   &f.P,     &f.Q,     &f.Fx,     &f.Fy,    &f.Gx,   &f.Gy,    &f.A,     &f.B,
                &f.C,     &f.E,     &f.Uxx,   &f.Vxy,   &f.Uxy,   &f.Vyy,   &f.DUxx,  &f.DVxy,
                &f.DUxy,  &f.DVyy,  &f.U4,    &f.V4,     &f.U1p,   &f.V1p,  &f.Udisp, &f.Vdisp, &f.ETAx,
                &f.ETAy,  &f.ETAT,  &f.AGE,   &f.AGEn,   &f.nu,    &f.SourceX, &f.SourceY, &f.WM, &f.Hmax};
    for (T **p : tf) *p = (T *)take(plane * sizeof(T));
    // statistics planes only when switched on
    if (g.track_hmin) f.Hmin = (T *)take(plane * sizeof(T));
    if (g.track_roller) {
        f.ROLLER = (T *)take(plane * sizeof(T));
        f.UNDERTOW_U = (T *)take(plane * sizeof(T));
        f.UNDERTOW_V = (T *)take(plane * sizeof(T));
    }
    if (g.track_umax) f.Umax = (T *)take(plane * sizeof(T));
    if (g.track_mfmax) f.MFmax = (T *)take(plane * sizeof(T));
    if (g.stats) {
        T **sf[] = {&f.ETAmean, &f.Umean, &f.Vmean, &f.ETAsum, &f.Usum, &f.Vsum, &f.ETA2sum, &f.ETA2mean,
                    &f.SigWH, &f.Emax, &f.Emin, &f.HavgSum, &f.HrmsSum, &f.WHave, &f.WHrms, &f.NZU};
        for (T **p : sf) *p = (T *)take(plane * sizeof(T));
        if (sizeof(T) == sizeof(float)) {
            T **kf[] = {&f.kETAsum, &f.kUsum, &f.kVsum, &f.kETA2sum};
            for (T **p : kf) *p = (T *)take(plane * sizeof(T));
        }
        if (g.track_rad)
            f.rad = (T *)take((size_t)(sizeof(T) == sizeof(double) ? fw::RP_N64 : fw::RP_N32) * plane * sizeof(T));
    }
    uint8_t **mf[] = {&f.MASK, &f.MASKn, &f.MASK9, &f.MASK_STRUC};
    for (uint8_t **p : mf) *p = (uint8_t *)take(plane);
    f.rhs_x = (T *)take(plane * sizeof(T));
    f.rhs_y = (T *)take(plane * sizeof(T));
    double **df[] = {&f.ty, &f.tp, &f.tq, &f.tc};
    for (double **p : df) *p = (double *)take(plane * sizeof(double));
    f.DepthD = sizeof(T) == sizeof(double) ? (double *)f.Depth : (double *)take(plane * sizeof(double));
    f.m9_dirty = (int *)take(sizeof(int));
    f.sw_p[0] = f.tp;
    f.sw_q[0] = f.tq;
    f.sw_c[0] = f.tc;
    f.sw_p[1] = f.sw_q[1] = f.sw_c[1] = nullptr;
    if (sizeof(T) == sizeof(float)) {
        // y factors in the same launch as x: a scratch of its own
        f.sw_p[1] = (double *)take(plane * sizeof(double));
        f.sw_q[1] = (double *)take(plane * sizeof(double));
        f.sw_c[1] = (double *)take(plane * sizeof(double));
        for (int d = 0; d < 2; d++) {
            float **ff[] = {&f.fac_it[d], &f.fac_A[d], &f.fac_lr[d], &f.fac_cp[d], &f.fac_p[d],
                            &f.fac_q[d], &f.fac_ah[d], &f.fac_al[d], &f.fac_ch[d], &f.fac_cl[d]};
            for (float **p : ff) *p = (float *)take(plane * sizeof(float));
            const LinePart &lp = d == 0 ? c->px : c->py;
            // per line: 2P reduced rows x 3 + P chunks x 2 + 2P second solution + 3
            const size_t per_line = (size_t)2 * lp.P * 3 + (size_t)lp.P * 2 + (size_t)2 * lp.P + 3;
            f.fac_red[d] = (float *)take((size_t)lp.nlines * per_line * sizeof(float));
        }
    }
    // the two directions' factorisation rows side by side (both directions
    // are factored in one launch); the per-stage solves reuse the start
    const size_t nred = (size_t)c->px.nlines * 2 * c->px.P + (size_t)c->py.nlines * 2 * c->py.P;
    f.red = (double *)take(nred * 6 * sizeof(double));
    f.dsc = (double *)take(S_NSLOT * sizeof(double));
    f.fsc = (float *)take(FS_NSLOT * sizeof(float));
    f.dtmin_bits = (unsigned long long *)take(sizeof(unsigned long long));
    f.etamax_bits = (unsigned long long *)take(sizeof(unsigned long long));
    f.ncand = (int *)take(sizeof(int));
    f.cand = (int *)take((size_t)c->ncand_cap * sizeof(int));
    const int nf = c->p.wavemaker == FW_WK_JON_2D ? (c->p.nfreq > 0 ? c->p.nfreq : 1) : 1;
    f.omega = (double *)take((size_t)nf * sizeof(double));
    f.wmcs = (double *)take((size_t)nf * 2 * sizeof(double));
    f.wmcsf = (float *)take((size_t)nf * 2 * sizeof(float));
    f.Cm = f.Sm = nullptr;  // band tables are allocated by fw_init
    void *stg = take((size_t)(g.Mloc + 1) * (size_t)(g.Nloc + 1) * sizeof(double));
    if (assign) {
        c->F<T>() = f;
        c->staging = stg;
    }
    return off;
}

int upload_array(fw_ctx *c, void *dst, const void *src, size_t bytes) {
    cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    return cuda_status(c, e);
}

double *dsc_ptr(fw_ctx *c) { return c->p.precision == FW_PREC_FP64 ? c->fd.dsc : c->ff.dsc; }

template <typename T> void dispatch_stage(fw_ctx *c, int istage) { launch_stage<T>(c, istage); }

// one whole step on the stream (main.F:284-535 minus OUTPUT)
template <typename T> void enqueue_step(fw_ctx *c) {
    launch_begin_step<T>(c);
    for (int s = 1; s <= 3; s++) launch_stage<T>(c, s);
    launch_end_step<T>(c);
}

int check_ready(fw_ctx *c) {
    if (!c) return FW_ERR_BAD_PARAM;
    if (!c->initialized) return FW_ERR_NOT_READY;
    if (c->sticky_error) return FW_ERR_CUDA;
    return FW_OK;
}

int finish(fw_ctx *c) {
    cudaError_t e = cudaGetLastError();
    return cuda_status(c, e);
}

unsigned long long *etamax_ptr(fw_ctx *c) {
    return c->p.precision == FW_PREC_FP64 ? c->fd.etamax_bits : c->ff.etamax_bits;
}

template <typename T> void save_pingpong(fw_ctx *c, void **p) {
    fw::Fields<T> &f = c->F<T>();
    p[0] = f.MASK;
    p[1] = f.MASKn;
    p[2] = f.AGE;
    p[3] = f.AGEn;
}

template <typename T> void load_pingpong(fw_ctx *c, void *const *p) {
    fw::Fields<T> &f = c->F<T>();
    f.MASK = (uint8_t *)p[0];
    f.MASKn = (uint8_t *)p[1];
    f.AGE = (T *)p[2];
    f.AGEn = (T *)p[3];
}

// host pointer state that a captured graph bakes in
long long swap_state(fw_ctx *c) {
    if (c->p.precision == FW_PREC_FP64) return (long long)((uintptr_t)c->fd.MASK ^ ((uintptr_t)c->fd.AGE << 1));
    return (long long)((uintptr_t)c->ff.MASK ^ ((uintptr_t)c->ff.AGE << 1));
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against the driver library)
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn encode_fn() {
    static EncodeTiledFn fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeTiledFn)p;
        else
            cudaGetLastError();
    }
    return fn;
}

// the flux kernels' tensor maps (fw::FluxMaps): a plane of pitch x (Nloc+1)
// elements, boxes 40 (fields) or 48 (MASK) cells wide and as high as the
// tile's staged rows; zero outside the plane
template <typename T> bool build_flux_maps(fw_ctx *c) {
    EncodeTiledFn enc = encode_fn();
    if (!enc) return false;
    fw::Fields<T> &f = c->F<T>();
    const Grid &g = c->g;
    T *fld[7] = {f.U, f.V, f.HU, f.HV, f.Eta, f.U4, f.V4};
    uint8_t *mb[2] = {f.MASK, f.MASKn};
    const cuuint64_t dims[2] = {(cuuint64_t)g.pitch, (cuuint64_t)(g.Nloc + 1)};
    const cuuint64_t st_f[1] = {(cuuint64_t)g.pitch * sizeof(T)}, st_m[1] = {(cuuint64_t)g.pitch};
    const cuuint32_t es[2] = {1, 1};
    const CUtensorMapDataType dt = sizeof(T) == sizeof(double) ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64
                                                               : CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
    for (int dir = 0; dir < 2; dir++)
        for (int fi = 0; fi < fw::FLUX_FY_N; fi++) {
            const int fy = 8 << fi;
            if (sizeof(T) == sizeof(double) && fy == 32) continue;
            const cuuint32_t bh = (cuuint32_t)(dir == 0 ? fy : fy + 6);
            const cuuint32_t box_f[2] = {40, bh}, box_m[2] = {48, bh};
            for (int mi = 0; mi < 2; mi++) {
                fw::FluxMaps &m = c->fmaps[dir][fi][mi];
                for (int v = 0; v < 7; v++)
                    if (enc(&m.m[v], dt, 2, fld[v], dims, st_f, box_f, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                            CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
                        return false;
                if (enc(&m.m[7], CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, mb[mi], dims, st_m, box_m, es,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
                    return false;
            }
        }
    c->fmask_base[0] = f.MASK;
    c->fmask_base[1] = f.MASKn;
    return fw::flux_tma_attrs<T>();
}

// launch-shape candidates of the per-cell kernels (bx a multiple of 32,
// at most 256 threads, as the kernels' launch bounds allow)
const int CELL_CANDIDATES[][2] = {{32, 8}, {32, 4}, {32, 2}, {64, 4}, {64, 2}, {128, 2}, {128, 1}, {256, 1}};
const char *const TUNE_NAMES[fw::TK_N] = {"disp_a", "disp_b", "update", "post_mask_break", "maskmul"};
std::mutex tune_mu;
std::map<std::array<long long, 8>, std::array<int, FW_TUNE_LEN>> tune_cache;

bool tune_valid(const fw_ctx *c, const int *t) {
    for (int k = 0; k < fw::TK_N; k++) {
        const int bx = t[2 * k], by = t[2 * k + 1];
        if (bx < 32 || bx % 32 != 0 || by < 1 || bx * by > 256) return false;
    }
    const bool fp64 = c->p.precision == FW_PREC_FP64;
    for (int d = 0; d < 2; d++) {
        const int fy = t[fw::TUNE_FLUX + d];
        if (fy != 8 && fy != 16 && (fp64 || fy != 32)) return false;
        const int tma = t[fw::TUNE_FLUX_TMA + d];
        if (tma != 0 && tma != 1) return false;
        if (tma == 1 && !c->fmaps_ok) return false;
    }
    return true;
}

// average ms of a launch of one named kernel: two warm-up launches, then
// eight timed with CUDA events on the context stream; e records a failure
double time_named(fw_ctx *c, bool fp64, const char *name, cudaError_t &e) {
    cudaEvent_t a = nullptr, b = nullptr;
    double ms_out = 1e30;
    if ((e = cudaEventCreate(&a)) != cudaSuccess || (e = cudaEventCreate(&b)) != cudaSuccess) {
        if (a) cudaEventDestroy(a);
        return ms_out;
    }
    auto launch = [&]() { return fp64 ? fw::launch_by_name<double>(c, name) : fw::launch_by_name<float>(c, name); };
    constexpr int NREP = 8;
    for (int k = 0; k < 2; k++) launch();
    e = cudaEventRecord(a, c->stream);
    for (int k = 0; k < NREP && e == cudaSuccess; k++) launch();
    if (e == cudaSuccess) e = cudaEventRecord(b, c->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(b);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
    if (e == cudaSuccess && c->sticky_error) e = (cudaError_t)c->sticky_error;
    if (e == cudaSuccess) ms_out = (double)ms / NREP;
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return ms_out;
}

// Every field and device scalar to zero, the CFL minimum to +inf: the
// state of a new context, which fw_init also starts from, so that a context
// initialised again runs like a new one (nothing of an earlier run, such as
// a NaN in a face flux, survives).
cudaError_t clear_arena(fw_ctx *c) {
    cudaError_t e = cudaMemsetAsync(c->arena, 0, c->arena_bytes, c->stream);
    const unsigned long long inf_bits = 0x7ff0000000000000ull;
    unsigned long long *dtb = c->p.precision == FW_PREC_FP64 ? c->fd.dtmin_bits : c->ff.dtmin_bits;
    if (e == cudaSuccess) e = cudaMemcpyAsync(dtb, &inf_bits, sizeof(inf_bits), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    return e;
}

int read_status(fw_ctx *c, int *status) {
    unsigned long long bits = 0;
    cudaError_t e = cudaMemcpyAsync(&bits, etamax_ptr(c), sizeof(bits), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_status(c, e);
    double mx;
    std::memcpy(&mx, &bits, sizeof(mx));
    int st = FW_OK;
    if (!(mx == mx) || std::isinf(mx)) st = FW_ERR_NAN;
    else if (mx > c->EtaBlowVal) st = FW_ERR_BLOWUP;
    if (status) *status = st;
    return FW_OK;
}

}  // namespace

extern "C" {

void fw_params_default(fw_params *p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->Mglob = 0;
    p->Nglob = 0;
    p->DX = 1.0;
    p->DY = 1.0;
    p->periodic = 0;
    p->dispersion = 1;
    p->gamma1 = 1.0;
    p->gamma2 = 1.0;
    p->gamma3 = 1.0;
    p->beta_ref = -0.531;
    p->viscosity_breaking = 1;
    p->show_breaking = 1;
    p->cbrk1 = 0.65;
    p->cbrk2 = 0.35;
    p->wavemaker_cbrk = 1.0;
    p->nu_bkg = 0.0;
    p->swe_eta_dep = 0.80;
    p->cfl = 0.5;
    p->froude_cap = 3.0;
    p->min_depth = 0.1;
    p->min_depth_frc = 0.1;
    p->trough_limit = -999999.0;
    p->crest_limit = 999999.0;
    p->r_sponge = 0.85;
    p->a_sponge = 5.0;
    p->wavemaker = FW_WK_NONE;
    p->delta_wk = 0.5;
    p->time_ramp = 0.0;
    p->ywidth_wk = 999999.0;
    p->sigma_theta = 10.0;
    p->spreading = FW_SPREAD_WRAPPED_NORMAL;
    p->precision = FW_PREC_FP64;
    p->device = 0;
    p->steady_time = 999999.0;  // LARGE: no time means
    p->t_intv_mean = 999999.0;
}

const char *fw_strerror(int s) {
    if (s > 0 || s < -10) return "unknown status";
    return kErrText[-s];
}

int fw_create(const fw_params *p, fw_ctx **out) {
    if (!p || !out) return FW_ERR_BAD_PARAM;
    *out = nullptr;
    if (p->Mglob < 2 || p->Nglob < 2 || !(p->DX > 0) || !(p->DY > 0) || !(p->cfl > 0) ||
        (p->precision != FW_PREC_FP64 && p->precision != FW_PREC_MIXED) ||
        (p->wavemaker < FW_WK_NONE || p->wavemaker > FW_WK_JON_2D) || !(p->min_depth_frc > 0))
        return FW_ERR_BAD_PARAM;
    {
        // the kernels index a plane with 32-bit offsets: a plane (padded
        // rows of Mloc+1 cells, Nloc+1 rows) must hold fewer than 2^31
        // elements
        const long long pitch = ((long long)p->Mglob + 2 * NG + 1 + 31) / 32 * 32;
        if (pitch * ((long long)p->Nglob + 2 * NG + 1) >= (1ll << 31)) return FW_ERR_UNSUPPORTED;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= p->device) {
        cudaGetLastError();
        return FW_ERR_NO_DEVICE;
    }
    if (cudaSetDevice(p->device) != cudaSuccess) return FW_ERR_NO_DEVICE;
    fw_ctx *c = new (std::nothrow) fw_ctx();
    if (!c) return FW_ERR_OOM;
    c->p = *p;
    if (p->precision == FW_PREC_FP64) c->tune[fw::TUNE_FLUX + 1] = 16;
    Grid &g = c->g;
    std::memset(&g, 0, sizeof(g));
    g.Mglob = p->Mglob;
    g.Nglob = p->Nglob;
    g.Mloc = p->Mglob + 2 * NG;
    g.Nloc = p->Nglob + 2 * NG;
    g.pitch = ((g.Mloc + 1) + 31) / 32 * 32;
    g.ib = NG;
    g.ie = g.Mloc - NG - 1;
    g.jb = NG;
    g.je = g.Nloc - NG - 1;
    g.periodic = p->periodic;
    g.dispersion = p->dispersion;
    g.visc_breaking = p->viscosity_breaking;
    g.show_breaking = p->show_breaking;
    g.direct_sponge = p->direct_sponge;
    g.friction_sponge = p->friction_sponge;
    g.eta_limiter = p->eta_limiter;
    g.wavemaker = p->wavemaker;
    g.nfreq = p->wavemaker == FW_WK_JON_2D ? p->nfreq : 0;
    g.DX = p->DX;
    g.DY = p->DY;
    // dispersion coefficients (init.F:656-664); Gamma1/2 off without dispersion
    g.gamma1 = p->dispersion ? p->gamma1 : 0.0;
    g.gamma2 = p->dispersion ? p->gamma2 : 0.0;
    g.has_g2 = g.gamma2 > 0.0 ? 1 : 0;
    g.track_hmin = p->track_hmin;
    g.track_roller = p->track_roller;
    g.track_rad = p->track_radiation && p->steady_time < 999999.0 ? 1 : 0;
    g.brk_passes = 8;
    g.track_umax = p->track_umax;
    g.track_mfmax = p->track_mfmax;
    g.steady_time = p->steady_time;
    g.t_intv_mean = p->t_intv_mean;
    g.stats = p->steady_time < 999999.0 ? 1 : 0;  // MIXING_STUFF can run
    g.gamma3 = p->gamma3;
    g.b1 = p->beta_ref * p->beta_ref;
    g.b2 = p->beta_ref;
    g.Beta_1 = p->beta_ref + 1.0;
    g.Beta_2 = (1.0 / 5.0) * (1.0 / 5.0) / 1.0;
    g.cbrk1 = p->cbrk1;
    g.cbrk2 = p->cbrk2;
    g.wavemaker_cbrk = p->wavemaker_cbrk;
    g.nu_bkg = p->nu_bkg;
    g.swe_eta_dep = p->swe_eta_dep;
    g.froude_cap = p->froude_cap;
    g.min_depth_frc = p->min_depth_frc;
    g.cfl = p->cfl;
    g.fixed_dt = p->fixed_dt;
    g.dt_fixed = p->dt_fixed;
    g.trough = p->trough_limit;
    g.crest = p->crest_limit;
    g.xc_wk = p->xc_wk;
    g.yc_wk = p->yc_wk;
    g.ywidth_wk = p->ywidth_wk;
    g.tperiod = p->tperiod;
    g.time_ramp = p->time_ramp;
    g.freq_peak = p->freq_peak;
    g.ilo = 1;
    g.ihi = 0;
    g.jlo = 1;
    g.jhi = 0;
    for (int d = 0; d < 2; d++) {
        const double h = d == 0 ? p->DX : p->DY;
        g.cA[d] = g.b1 / 2.0 / (h * h);
        g.cB[d] = g.b2 / (h * h);
        g.cC[d] = (-g.b1 - 2.0 * g.b2) / (h * h);
        // the FP64 path's constant sub-expressions of etauv_solver.F:406-409
        // and 504-507, evaluated left to right as there (IEEE division gives
        // the device's value)
        g.tK1[d] = g.b1 / 2.0 / h / h;
        g.tK2[d] = g.b2 / h / h;
        g.tK3[d] = -g.b1 / h / h;
        g.tK4[d] = 2.0 * g.b2 / h / h;
    }
    g.rdx = 1.0 / p->DX;
    g.rdy = 1.0 / p->DY;
    fill_float_constants(g);
    c->px = make_part(p->Mglob, p->Nglob);
    c->py = make_part(p->Nglob, p->Mglob);
    c->px.red0 = 0;
    c->py.red0 = (long long)c->px.nlines * 2 * c->px.P * 6;
    c->ncand_cap = (p->Mglob + 2) * (p->Nglob + 2);
    // the factored solve assumes tmp2 = 1 + Gamma1*MASK9*(-b1-2*b2)/h^2*dep^2
    // never vanishes, which holds for -b1-2*b2 >= 0 (Beta_ref in [-2, 0])
    c->factored = (p->precision == FW_PREC_MIXED) && (-g.b1 - 2.0 * g.b2 >= 0.0) ? 1 : 0;
    const bool fp64 = p->precision == FW_PREC_FP64;
    const size_t bytes = fp64 ? carve<double>(c, nullptr, false) : carve<float>(c, nullptr, false);
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        delete c;
        return FW_ERR_CUDA;
    }
    if (cudaMalloc(&c->arena, bytes) != cudaSuccess) {
        cudaGetLastError();
        cudaStreamDestroy(c->stream);
        delete c;
        return FW_ERR_OOM;
    }
    c->arena_bytes = bytes;
    if (fp64) carve<double>(c, (char *)c->arena, true);
    else carve<float>(c, (char *)c->arena, true);
    // the TMA-staged flux kernels are a tuning choice; without their maps
    // the load-based kernels run
    c->fmaps_ok = (fp64 ? build_flux_maps<double>(c) : build_flux_maps<float>(c)) ? 1 : 0;
    cudaGetLastError();
    cudaError_t e = clear_arena(c);
    if (e != cudaSuccess) {
        cudaGetLastError();
        fw_destroy(c);
        return FW_ERR_CUDA;
    }
    *out = c;
    return FW_OK;
}

int fw_destroy(fw_ctx *c) {
    if (!c) return FW_ERR_BAD_PARAM;
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->out_stream) cudaStreamSynchronize(c->out_stream);
    if (c->graph) cudaGraphExecDestroy(c->graph);
    for (cudaGraphExec_t g1 : c->graph1)
        if (g1) cudaGraphExecDestroy(g1);
    if (c->out_buf) cudaFree(c->out_buf);
    if (c->in_buf) cudaFree(c->in_buf);
    for (cudaEvent_t ev : c->in_ev)
        if (ev) cudaEventDestroy(ev);
    if (c->out_ready) cudaEventDestroy(c->out_ready);
    if (c->out_done) cudaEventDestroy(c->out_done);
    if (c->out_stream) cudaStreamDestroy(c->out_stream);
    void *band[4] = {(void *)c->fd.Cm, (void *)c->fd.Sm, (void *)c->ff.Cm, (void *)c->ff.Sm};
    for (void *b : band)
        if (b) cudaFree(b);
    if (c->arena) cudaFree(c->arena);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return FW_OK;
}

int fw_init(fw_ctx *c, const double *depth, const double *eta, const double *u, const double *v,
            const double *phases) {
    if (!c) return FW_ERR_BAD_PARAM;
    HostCase hc;
    std::string err;
    int rc = build_case(c->p, depth, eta, u, v, phases, hc, err);
    if (rc != FW_OK) return rc;
    cudaError_t ce = clear_arena(c);
    if (ce != cudaSuccess) return cuda_status(c, ce);
    Grid &g = c->g;
    g.T_brk = hc.T_brk;
    g.width_wk = hc.Width_WK;
    g.D_gen = hc.D_gen;
    g.beta_gen = hc.beta_gen;
    g.rlamda = hc.rlamda;
    c->EtaBlowVal = hc.EtaBlowVal;
    fill_float_constants(g);
    if (hc.ilo <= hc.ihi && hc.jlo <= hc.jhi) {
        g.ilo = hc.ilo - 1;
        g.ihi = hc.ihi - 1;
        g.jlo = hc.jlo - 1;
        g.jhi = hc.jhi - 1;
    } else {
        g.ilo = 1;
        g.ihi = 0;
        g.jlo = 1;
        g.jhi = 0;
    }
    struct {
        const char *n;
        const void *d;
    } up[] = {{"Depth", hc.Depth.data()}, {"Depthx", hc.Depthx.data()}, {"Depthy", hc.Depthy.data()},
              {"Eta", hc.Eta.data()},     {"U", hc.U.data()},           {"V", hc.V.data()},
              {"H", hc.H.data()},         {"HU", hc.HU.data()},         {"HV", hc.HV.data()},
              {"Ubar", hc.Ubar.data()},   {"Vbar", hc.Vbar.data()},     {"Cd", hc.Cd.data()},
              {"SPONGE", hc.SPONGE.data()}, {"nu_break", hc.nu.data()}, {"MASK", hc.MASK.data()},
              {"MASK9", hc.MASK9.data()}, {"MASK_STRUC", hc.MASK_STRUC.data()}};
    for (auto &x : up) {
        rc = put_named(c, x.n, x.d);
        if (rc != FW_OK) return rc;
    }
    // JON_2D band tables
    const int bw = hc.ihi - hc.ilo + 1, bh = hc.jhi - hc.jlo + 1;
    if (c->p.wavemaker == FW_WK_JON_2D && bw > 0 && bh > 0) {
        // the band Cm/Sm in the field precision (the mixed path sums them in
        // float), computed on the device from the spectrum tables
        const bool d = c->p.precision == FW_PREC_FP64;
        const size_t es = d ? sizeof(double) : sizeof(float);
        const size_t mf = c->p.nfreq, mt = c->p.ntheta;
        const size_t nb = (size_t)bw * bh * mf * es;
        void *Cm = nullptr, *Sm = nullptr;
        double *tab = nullptr;
        const size_t ntab = 3 * mf * mt + mf;
        if (cudaMalloc(&Cm, nb) != cudaSuccess || cudaMalloc(&Sm, nb) != cudaSuccess ||
            cudaMalloc(&tab, ntab * sizeof(double)) != cudaSuccess) {
            cudaGetLastError();
            if (Cm) cudaFree(Cm);
            if (Sm) cudaFree(Sm);
            return FW_ERR_OOM;
        }
        void *oldc = d ? (void *)c->fd.Cm : (void *)c->ff.Cm, *olds = d ? (void *)c->fd.Sm : (void *)c->ff.Sm;
        if (oldc) cudaFree(oldc);
        if (olds) cudaFree(olds);
        std::vector<double> h(ntab);
        std::copy(hc.jon_dgen.begin(), hc.jon_dgen.end(), h.begin());
        std::copy(hc.jon_rlamda.begin(), hc.jon_rlamda.end(), h.begin() + mf * mt);
        std::copy(hc.jon_phases.begin(), hc.jon_phases.end(), h.begin() + 2 * mf * mt);
        std::copy(hc.jon_betagen.begin(), hc.jon_betagen.end(), h.begin() + 3 * mf * mt);
        rc = upload_array(c, tab, h.data(), ntab * sizeof(double));
        const int i0 = hc.ilo - (NG + 1), j0 = hc.jlo - (NG + 1);  // I-Ibeg, J-Jbeg of the band's first cell
        if (d) {
            c->fd.Cm = (double *)Cm;
            c->fd.Sm = (double *)Sm;
            if (rc == FW_OK) launch_cm_sm<double>(c, bw, bh, i0, j0, tab, c->fd.Cm, c->fd.Sm);
        } else {
            c->ff.Cm = (float *)Cm;
            c->ff.Sm = (float *)Sm;
            if (rc == FW_OK) launch_cm_sm<float>(c, bw, bh, i0, j0, tab, c->ff.Cm, c->ff.Sm);
        }
        cudaError_t e = cudaStreamSynchronize(c->stream);
        cudaFree(tab);
        if (rc != FW_OK) return rc;
        if (e != cudaSuccess) return cuda_status(c, e);
        double *om = c->p.precision == FW_PREC_FP64 ? c->fd.omega : c->ff.omega;
        if ((rc = upload_array(c, om, hc.omega.data(), hc.omega.size() * sizeof(double))) != FW_OK) return rc;
    }
    double sc[S_NSLOT] = {0};
    if ((rc = upload_array(c, dsc_ptr(c), sc, sizeof(sc))) != FW_OK) return rc;
    const int one = 1;  // factor the tridiagonal matrices at the first stage
    int *dirty = c->p.precision == FW_PREC_FP64 ? c->fd.m9_dirty : c->ff.m9_dirty;
    if ((rc = upload_array(c, dirty, &one, sizeof(one))) != FW_OK) return rc;
    if (c->graph) {
        cudaGraphExecDestroy(c->graph);
        c->graph = nullptr;
    }
    c->invalidate_graphs();
    c->initialized = 1;
    return FW_OK;
}

int fw_get_field(fw_ctx *c, const char *name, void *host) {
    if (!c || !name || !host) return FW_ERR_BAD_PARAM;
    FieldRef r;
    if (c->p.precision == FW_PREC_FP64) {
        if (!find_field<double>(c, name, r)) return FW_ERR_BAD_PARAM;
        return get_field<double>(c, r, host);
    }
    if (!find_field<float>(c, name, r)) return FW_ERR_BAD_PARAM;
    return get_field<float>(c, r, host);
}

int fw_set_field(fw_ctx *c, const char *name, const void *host) {
    if (!c || !name || !host) return FW_ERR_BAD_PARAM;
    return put_named(c, name, host);
}

// REAL(SP) host arrays: the mixed build's float fields move with one 2-D
// copy each way; the FP64 build's go through the staging plane and a
// conversion kernel.  Masks keep their int32 transfers (fw_get_field).
int fw_get_field_f32(fw_ctx *c, const char *name, float *host) {
    if (!c || !name || !host) return FW_ERR_BAD_PARAM;
    const bool fp64 = c->p.precision == FW_PREC_FP64;
    FieldRef r;
    if (!(fp64 ? find_field<double>(c, name, r) : find_field<float>(c, name, r)) || r.is_mask)
        return FW_ERR_BAD_PARAM;
    int w, h;
    extent(c, r.kind, w, h);
    cudaError_t e;
    if (fp64) {
        convert_out_f32(c, (const double *)r.ptr, (float *)c->staging, w, h);
        e = cudaMemcpyAsync(host, c->staging, (size_t)w * h * sizeof(float), cudaMemcpyDeviceToHost, c->stream);
    } else {
        e = cudaMemcpy2DAsync(host, (size_t)w * sizeof(float), r.ptr, (size_t)c->g.pitch * sizeof(float),
                              (size_t)w * sizeof(float), (size_t)h, cudaMemcpyDeviceToHost, c->stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    return cuda_status(c, e);
}

int fw_set_field_f32(fw_ctx *c, const char *name, const float *host) {
    if (!c || !name || !host) return FW_ERR_BAD_PARAM;
    const bool fp64 = c->p.precision == FW_PREC_FP64;
    FieldRef r;
    if (!(fp64 ? find_field<double>(c, name, r) : find_field<float>(c, name, r)) || r.is_mask)
        return FW_ERR_BAD_PARAM;
    int w, h;
    extent(c, r.kind, w, h);
    cudaError_t e;
    if (fp64) {
        e = cudaMemcpyAsync(c->staging, host, (size_t)w * h * sizeof(float), cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess) convert_in_f32(c, (const float *)c->staging, (double *)r.ptr, w, h);
    } else {
        e = cudaMemcpy2DAsync(r.ptr, (size_t)c->g.pitch * sizeof(float), host, (size_t)w * sizeof(float),
                              (size_t)w * sizeof(float), (size_t)h, cudaMemcpyHostToDevice, c->stream);
        // the double Depth of the total-depth tests, widened from the floats
        if (e == cudaSuccess && std::strcmp(name, "Depth") == 0) {
            e = cudaMemcpyAsync(c->staging, host, (size_t)w * h * sizeof(float), cudaMemcpyHostToDevice, c->stream);
            if (e == cudaSuccess) convert_in_f32(c, (const float *)c->staging, c->ff.DepthD, w, h);
        }
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    return cuda_status(c, e);
}

int fw_get_points(fw_ctx *c, const char *name, int n, const int *I, const int *J, double *out) {
    int rc = check_ready(c);
    if (rc != FW_OK) return rc;
    if (!name || n < 0 || (n > 0 && (!I || !J || !out))) return FW_ERR_BAD_PARAM;
    if (n == 0) return FW_OK;
    FieldRef r;
    const bool d = c->p.precision == FW_PREC_FP64;
    if (!(d ? find_field<double>(c, name, r) : find_field<float>(c, name, r))) return FW_ERR_BAD_PARAM;
    int w, h;
    extent(c, r.kind, w, h);
    // offsets, then the gathered values, in the staging plane
    const size_t cap = (size_t)c->g.pitch * (size_t)(c->g.Nloc + 1) * sizeof(double);
    if ((size_t)n * (sizeof(int) + sizeof(double)) + 16 > cap) return FW_ERR_BAD_PARAM;
    std::vector<int> off((size_t)n);
    for (int k = 0; k < n; k++) {
        if (I[k] < 1 || I[k] > w || J[k] < 1 || J[k] > h) return FW_ERR_BAD_PARAM;
        off[k] = (I[k] - 1) + (J[k] - 1) * c->g.pitch;
    }
    int *d_off = (int *)c->staging;
    double *d_out = (double *)((char *)c->staging + (((size_t)n * sizeof(int) + 15) / 16) * 16);
    cudaError_t e = cudaMemcpyAsync(d_off, off.data(), (size_t)n * sizeof(int), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) {
        gather_points(c, r.ptr, r.is_mask ? 2 : (d ? 0 : 1), d_off, n, d_out);
        e = cudaMemcpyAsync(out, d_out, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    return cuda_status(c, e);
}

int fw_get_scalar(fw_ctx *c, const char *name, double *v) {
    if (!c || !name || !v) return FW_ERR_BAD_PARAM;
    if (!std::strcmp(name, "TIME") || !std::strcmp(name, "DT") || !std::strcmp(name, "T_sum") ||
        !std::strcmp(name, "ICOUNT_MEAN")) {
        double sc[S_NSLOT];
        cudaError_t e = cudaMemcpyAsync(sc, dsc_ptr(c), sizeof(sc), cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) return cuda_status(c, e);
        *v = !std::strcmp(name, "TIME") ? sc[S_TIME]
             : !std::strcmp(name, "DT") ? sc[S_DT]
             : !std::strcmp(name, "T_sum") ? sc[S_TSUM]
                                            : sc[S_NMEAN];
        return FW_OK;
    }
    if (!std::strcmp(name, "EtaBlowVal")) *v = c->EtaBlowVal;
    else if (!std::strcmp(name, "T_brk")) *v = c->g.T_brk;
    else if (!std::strcmp(name, "Width_WK")) *v = c->g.width_wk;
    else if (!std::strcmp(name, "D_gen")) *v = c->g.D_gen;
    else if (!std::strcmp(name, "beta_gen")) *v = c->g.beta_gen;
    else if (!std::strcmp(name, "rlamda")) *v = c->g.rlamda;
    else if (!std::strcmp(name, "ilo")) *v = c->g.ilo + 1;
    else if (!std::strcmp(name, "ihi")) *v = c->g.ihi + 1;
    else if (!std::strcmp(name, "jlo")) *v = c->g.jlo + 1;
    else if (!std::strcmp(name, "jhi")) *v = c->g.jhi + 1;
    else if (!std::strcmp(name, "pitch")) *v = c->g.pitch;
    else if (!std::strcmp(name, "WAIT_LIMIT")) *v = c->fmaps[0][0][0].wait_limit;
    else if (!std::strcmp(name, "BREAK_PASSES")) *v = c->g.brk_passes;
    else return FW_ERR_BAD_PARAM;
    return FW_OK;
}

int fw_set_scalar(fw_ctx *c, const char *name, double v) {
    if (!c || !name) return FW_ERR_BAD_PARAM;
    if (!std::strcmp(name, "TIME") || !std::strcmp(name, "DT")) {
        const int slot = !std::strcmp(name, "TIME") ? S_TIME : S_DT;
        cudaError_t e = cudaMemcpyAsync(dsc_ptr(c) + slot, &v, sizeof(double), cudaMemcpyHostToDevice, c->stream);
        // the mixed path's float copies of DT and 1/DT follow a set DT
        const float fdt[2] = {(float)v, (float)(1.0 / v)};
        if (e == cudaSuccess && slot == S_DT && c->p.precision != FW_PREC_FP64)
            e = cudaMemcpyAsync(c->ff.fsc + FS_DT, fdt, sizeof(fdt), cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        return cuda_status(c, e);
    }
    if (!std::strcmp(name, "EtaBlowVal")) c->EtaBlowVal = v;
    else if (!std::strcmp(name, "WAIT_LIMIT")) {
        if (!(v >= 0.0 && v <= 4294967295.0)) return FW_ERR_BAD_PARAM;
        for (auto &by_dir : c->fmaps)
            for (auto &by_fy : by_dir)
                for (auto &m : by_fy) m.wait_limit = (unsigned)v;
    } else if (!std::strcmp(name, "BREAK_PASSES")) {
        if (!(v >= 0.0 && v <= 1.0e6)) return FW_ERR_BAD_PARAM;
        c->g.brk_passes = (int)v;
    } else if (!std::strcmp(name, "T_brk")) {
        c->g.T_brk = v;
        fill_float_constants(c->g);
    } else return FW_ERR_BAD_PARAM;
    c->invalidate_graphs();
    return FW_OK;
}

#define DISPATCH(fn)                                                           \
    do {                                                                       \
        int rc_ = check_ready(c);                                              \
        if (rc_ != FW_OK) return rc_;                                          \
        if (c->p.precision == FW_PREC_FP64) fn<double>(c); else fn<float>(c);  \
        return finish(c);                                                      \
    } while (0)

int fw_begin_step(fw_ctx *c) { DISPATCH(launch_begin_step); }
int fw_exchange(fw_ctx *c) {
    int rc = check_ready(c);
    if (rc != FW_OK) return rc;
    if (c->p.precision == FW_PREC_FP64) launch_exchange<double>(c, false);
    else launch_exchange<float>(c, false);
    return finish(c);
}
int fw_estimate_dt(fw_ctx *c) { DISPATCH(launch_estimate_dt); }
int fw_cal_dispersion(fw_ctx *c) { DISPATCH(launch_dispersion); }
int fw_fluxes(fw_ctx *c) { DISPATCH(launch_fluxes); }
int fw_source_terms(fw_ctx *c) { DISPATCH(launch_sources_debug); }
int fw_update_mask(fw_ctx *c) { DISPATCH(launch_update_mask); }
int fw_wave_breaking(fw_ctx *c) { DISPATCH(launch_breaking); }
int fw_sponge_damping(fw_ctx *c) { DISPATCH(launch_sponge); }

int fw_estimate_huv(fw_ctx *c, int istage) {
    int rc = check_ready(c);
    if (rc != FW_OK) return rc;
    if (istage < 1 || istage > 3) return FW_ERR_BAD_PARAM;
    if (c->p.precision == FW_PREC_FP64) launch_estimate_huv<double>(c, istage);
    else launch_estimate_huv<float>(c, istage);
    return finish(c);
}

int fw_stage(fw_ctx *c, int istage) {
    int rc = check_ready(c);
    if (rc != FW_OK) return rc;
    if (istage < 1 || istage > 3) return FW_ERR_BAD_PARAM;
    if (c->p.precision == FW_PREC_FP64) launch_stage<double>(c, istage);
    else launch_stage<float>(c, istage);
    return finish(c);
}

int fw_end_step(fw_ctx *c, int *status) {
    int rc = check_ready(c);
    if (rc != FW_OK) return rc;
    cudaError_t e = cudaMemsetAsync(etamax_ptr(c), 0, sizeof(unsigned long long), c->stream);
    if (e != cudaSuccess) return cuda_status(c, e);
    if (c->p.precision == FW_PREC_FP64) launch_end_step<double>(c);
    else launch_end_step<float>(c);
    if ((rc = finish(c)) != FW_OK) return rc;
    return read_status(c, status);
}

// the work of nsteps whole steps on the context's stream, without waiting;
// reset_max restarts the CHECK_BLOWUP maximum that read_status reads
static int enqueue_steps(fw_ctx *c, int nsteps, bool reset_max) {
    cudaError_t e;
    if (reset_max) {
        e = cudaMemsetAsync(etamax_ptr(c), 0, sizeof(unsigned long long), c->stream);
        if (e != cudaSuccess) return cuda_status(c, e);
    }
    const bool fp64 = c->p.precision == FW_PREC_FP64;
    int left = nsteps;
    // a graph holds two steps, after which every ping-pong buffer is back in
    // its place; it is (re)captured whenever the host-side buffer state
    // differs from the one it was captured with
    while (left >= 2) {
        if (!c->graph_ready || c->graph_state != swap_state(c)) {
            if (c->graph) {
                cudaGraphExecDestroy(c->graph);
                c->graph = nullptr;
            }
            const long long st = swap_state(c);
            cudaGraph_t graph;
            e = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal);
            if (e != cudaSuccess) return cuda_status(c, e);
            for (int k = 0; k < 2; k++) {
                if (fp64) enqueue_step<double>(c);
                else enqueue_step<float>(c);
            }
            e = cudaStreamEndCapture(c->stream, &graph);
            if (e != cudaSuccess) return cuda_status(c, e);
            e = cudaGraphInstantiate(&c->graph, graph, 0);
            cudaGraphDestroy(graph);
            if (e != cudaSuccess) return cuda_status(c, e);
            c->graph_ready = 1;
            c->graph_state = st;
        }
        e = cudaGraphLaunch(c->graph, c->stream);
        if (e != cudaSuccess) return cuda_status(c, e);
        left -= 2;
    }
    if (left == 1) {
        // a one-step graph for the current orientation (a step flips it);
        // two are kept, so a loop of single steps replays them in turn
        const long long st = swap_state(c);
        int slot = -1;
        for (int k = 0; k < 2; k++)
            if (c->graph1[k] && c->graph1_ok[k] && c->graph1_state[k] == st) slot = k;
        if (slot < 0) {
            slot = !c->graph1_ok[0] ? 0 : !c->graph1_ok[1] ? 1 : c->graph1_next;
            c->graph1_next = slot ^ 1;
            if (c->graph1[slot]) {
                cudaGraphExecDestroy(c->graph1[slot]);
                c->graph1[slot] = nullptr;
            }
            c->graph1_ok[slot] = 0;
            cudaGraph_t graph;
            e = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal);
            if (e != cudaSuccess) return cuda_status(c, e);
            if (fp64) enqueue_step<double>(c);
            else enqueue_step<float>(c);
            e = cudaStreamEndCapture(c->stream, &graph);
            if (e != cudaSuccess) return cuda_status(c, e);
            e = cudaGraphInstantiate(&c->graph1[slot], graph, 0);
            cudaGraphDestroy(graph);
            if (e != cudaSuccess) return cuda_status(c, e);
            c->graph1_ok[slot] = 1;
            c->graph1_state[slot] = st;
            if (fp64) save_pingpong<double>(c, c->graph1_post[slot]);
            else save_pingpong<float>(c, c->graph1_post[slot]);
        }
        e = cudaGraphLaunch(c->graph1[slot], c->stream);
        if (e != cudaSuccess) return cuda_status(c, e);
        if (fp64) load_pingpong<double>(c, c->graph1_post[slot]);
        else load_pingpong<float>(c, c->graph1_post[slot]);
    }
    return finish(c);
}

int fw_step(fw_ctx *c, int nsteps, int *status) {
    int rc = check_ready(c);
    if (rc != FW_OK) return rc;
    if (nsteps < 0) return FW_ERR_BAD_PARAM;
    if (status) *status = FW_OK;
    if (nsteps == 0) return FW_OK;
    if ((rc = enqueue_steps(c, nsteps, true)) != FW_OK) return rc;
    return read_status(c, status);
}

int fw_step_async(fw_ctx *c, int nsteps) {
    int rc = check_ready(c);
    if (rc != FW_OK) return rc;
    if (nsteps < 0) return FW_ERR_BAD_PARAM;
    return enqueue_steps(c, nsteps, true);
}

int fw_step_wait(fw_ctx *c, int *status) {
    int rc = check_ready(c);
    if (rc != FW_OK) return rc;
    return read_status(c, status);
}

int fw_ensemble_step(fw_ctx *const *ctxs, int n, int nsteps, int *status) {
    if (!ctxs || n < 0 || nsteps < 0) return FW_ERR_BAD_PARAM;
    for (int k = 0; k < n; k++) {
        const int rc = check_ready(ctxs[k]);
        if (rc != FW_OK) return rc;
        if (status) status[k] = FW_OK;
    }
    // round robin, one two-step graph per context per pass, so that every
    // stream has work queued while the others run
    for (int done = 0; done < nsteps; done += 2) {
        const int now = std::min(2, nsteps - done);
        for (int k = 0; k < n; k++) {
            const int rc = enqueue_steps(ctxs[k], now, done == 0);
            if (rc != FW_OK) return rc;
        }
    }
    int first = FW_OK;
    for (int k = 0; k < n; k++) {
        const int rc = read_status(ctxs[k], status ? &status[k] : nullptr);
        if (rc != FW_OK && first == FW_OK) first = rc;
    }
    return first;
}

}  // extern "C"

namespace fw {
int enqueue_one_step(fw_ctx *c) {
    if (c->p.precision == FW_PREC_FP64) enqueue_step<double>(c);
    else enqueue_step<float>(c);
    c->graph_ready = 0;
    return finish(c);
}
int reset_step_max(fw_ctx *c) {
    return cuda_status(c, cudaMemsetAsync(etamax_ptr(c), 0, sizeof(unsigned long long), c->stream));
}
int step_status(fw_ctx *c, int *status) { return read_status(c, status); }
long long buffer_state(fw_ctx *c) { return swap_state(c); }
}  // namespace fw

struct fw_ensemble {
    std::vector<fw_ctx *> ctx;
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    std::vector<cudaEvent_t> ready;  // one per run: its stream's earlier work
    cudaGraphExec_t exec = nullptr;
    std::vector<long long> states;   // swap_state of each run at capture
    std::vector<std::array<int, FW_TUNE_LEN>> tunes;
};

namespace {

bool ens_stale(const fw_ensemble *e) {
    if (!e->exec) return true;
    for (size_t k = 0; k < e->ctx.size(); k++) {
        if (e->states[k] != swap_state(e->ctx[k])) return true;
        if (std::memcmp(e->tunes[k].data(), e->ctx[k]->tune, sizeof(e->ctx[k]->tune)) != 0) return true;
    }
    return false;
}

// one parent graph whose child nodes are the runs' two-step captures
int ens_build(fw_ensemble *e) {
    if (e->exec) {
        cudaGraphExecDestroy(e->exec);
        e->exec = nullptr;
    }
    cudaGraph_t parent = nullptr;
    cudaError_t err = cudaGraphCreate(&parent, 0);
    for (size_t k = 0; k < e->ctx.size() && err == cudaSuccess; k++) {
        fw_ctx *c = e->ctx[k];
        cudaGraph_t g = nullptr;
        err = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal);
        if (err != cudaSuccess) break;
        for (int s = 0; s < 2; s++) {
            if (c->p.precision == FW_PREC_FP64) enqueue_step<double>(c);
            else enqueue_step<float>(c);
        }
        err = cudaStreamEndCapture(c->stream, &g);
        if (err != cudaSuccess) break;
        cudaGraphNode_t node;
        err = cudaGraphAddChildGraphNode(&node, parent, nullptr, 0, g);
        cudaGraphDestroy(g);
        e->states[k] = swap_state(c);
        std::memcpy(e->tunes[k].data(), c->tune, sizeof(c->tune));
    }
    if (err == cudaSuccess) err = cudaGraphInstantiate(&e->exec, parent, 0);
    if (parent) cudaGraphDestroy(parent);
    if (err != cudaSuccess) {
        cudaGetLastError();
        e->exec = nullptr;
        return FW_ERR_CUDA;
    }
    return FW_OK;
}

}  // namespace

extern "C" {

int fw_ensemble_create(fw_ctx *const *ctxs, int n, fw_ensemble **out) {
    if (!ctxs || n <= 0 || !out) return FW_ERR_BAD_PARAM;
    *out = nullptr;
    for (int k = 0; k < n; k++) {
        const int rc = check_ready(ctxs[k]);
        if (rc != FW_OK) return rc;
    }
    fw_ensemble *e = new (std::nothrow) fw_ensemble();
    if (!e) return FW_ERR_OOM;
    e->ctx.assign(ctxs, ctxs + n);
    e->states.assign(n, 0);
    e->tunes.resize(n);
    e->ready.assign(n, nullptr);
    bool ok = cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking) == cudaSuccess &&
              cudaEventCreateWithFlags(&e->done, cudaEventDisableTiming) == cudaSuccess;
    for (int k = 0; k < n && ok; k++) ok = cudaEventCreateWithFlags(&e->ready[k], cudaEventDisableTiming) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        fw_ensemble_destroy(e);
        return FW_ERR_CUDA;
    }
    *out = e;
    return FW_OK;
}

int fw_ensemble_run(fw_ensemble *e, int nsteps, int *status) {
    if (!e || nsteps < 0) return FW_ERR_BAD_PARAM;
    const int n = (int)e->ctx.size();
    for (int k = 0; k < n; k++) {
        const int rc = check_ready(e->ctx[k]);
        if (rc != FW_OK) return rc;
        if (status) status[k] = FW_OK;
    }
    if (nsteps == 0) return FW_OK;
    cudaError_t err = cudaSuccess;
    if (nsteps >= 2) {
        if (ens_stale(e)) {
            const int rc = ens_build(e);
            if (rc != FW_OK) return rc;
        }
        // the runs' earlier work, then the reset of their step maxima
        for (int k = 0; k < n && err == cudaSuccess; k++) {
            err = cudaEventRecord(e->ready[k], e->ctx[k]->stream);
            if (err == cudaSuccess) err = cudaStreamWaitEvent(e->stream, e->ready[k], 0);
            if (err == cudaSuccess)
                err = cudaMemsetAsync(etamax_ptr(e->ctx[k]), 0, sizeof(unsigned long long), e->stream);
        }
        for (int s = 0; s + 2 <= nsteps && err == cudaSuccess; s += 2) err = cudaGraphLaunch(e->exec, e->stream);
        if (err == cudaSuccess) err = cudaEventRecord(e->done, e->stream);
        for (int k = 0; k < n && err == cudaSuccess; k++) err = cudaStreamWaitEvent(e->ctx[k]->stream, e->done, 0);
        if (err != cudaSuccess) {
            cudaGetLastError();
            return FW_ERR_CUDA;
        }
    }
    if (nsteps % 2) {
        for (int k = 0; k < n; k++) {
            const int rc = enqueue_steps(e->ctx[k], 1, nsteps == 1);
            if (rc != FW_OK) return rc;
        }
    }
    int first = FW_OK;
    for (int k = 0; k < n; k++) {
        const int rc = read_status(e->ctx[k], status ? &status[k] : nullptr);
        if (rc != FW_OK && first == FW_OK) first = rc;
    }
    return first;
}

int fw_ensemble_destroy(fw_ensemble *e) {
    if (!e) return FW_ERR_BAD_PARAM;
    if (e->stream) cudaStreamSynchronize(e->stream);
    if (e->exec) cudaGraphExecDestroy(e->exec);
    for (cudaEvent_t ev : e->ready)
        if (ev) cudaEventDestroy(ev);
    if (e->done) cudaEventDestroy(e->done);
    if (e->stream) cudaStreamDestroy(e->stream);
    delete e;
    return FW_OK;
}

int fw_sync(fw_ctx *c) {
    if (!c) return FW_ERR_BAD_PARAM;
    return cuda_status(c, cudaStreamSynchronize(c->stream));
}

// ---------------------------------------------------------------------------
// Checkpoint / restore of the whole run state.  The reference restarts from
// written output fields (HOT_START, mod_global.F:387, io.F:805, main.F:189);
// a checkpoint here holds every device byte the step reads instead (the
// arena: fields, factorisation, device scalars, statistics, Kahan terms),
// the orientation of the MASK and AGE ping-pong buffers, the JON_2D band
// tables, EtaBlowVal and the host-side Grid, so that a restored run goes on
// bit for bit as the saved one would have.
// ---------------------------------------------------------------------------
}  // extern "C"
namespace {

const char kCkMagic[8] = {'F', 'W', 'C', 'K', 'P', 'T', '0', '1'};

struct CkHeader {
    char magic[8];
    uint32_t sizeof_params, sizeof_grid;
    int32_t precision, pad;
    uint64_t arena_bytes, band_bytes;  // band_bytes: each of Cm and Sm
    int64_t off_mask, off_maskn, off_age, off_agen;
    double EtaBlowVal;
};

// the fields of fw_params a restore requires to agree (all but device)
bool same_params(const fw_params &a, const fw_params &b) {
#define FW_SAME(x) (a.x == b.x)
    return FW_SAME(Mglob) && FW_SAME(Nglob) && FW_SAME(DX) && FW_SAME(DY) && FW_SAME(periodic) &&
           FW_SAME(dispersion) && FW_SAME(gamma1) && FW_SAME(gamma2) && FW_SAME(gamma3) && FW_SAME(beta_ref) &&
           FW_SAME(viscosity_breaking) && FW_SAME(show_breaking) && FW_SAME(cbrk1) && FW_SAME(cbrk2) &&
           FW_SAME(wavemaker_cbrk) && FW_SAME(nu_bkg) && FW_SAME(swe_eta_dep) && FW_SAME(cfl) && FW_SAME(fixed_dt) &&
           FW_SAME(dt_fixed) && FW_SAME(froude_cap) && FW_SAME(min_depth) && FW_SAME(min_depth_frc) &&
           FW_SAME(eta_limiter) && FW_SAME(trough_limit) && FW_SAME(crest_limit) && FW_SAME(direct_sponge) &&
           FW_SAME(sponge_west) && FW_SAME(sponge_east) && FW_SAME(sponge_south) && FW_SAME(sponge_north) &&
           FW_SAME(r_sponge) && FW_SAME(a_sponge) && FW_SAME(friction_sponge) && FW_SAME(cd_fixed) &&
           FW_SAME(wavemaker) && FW_SAME(amp_wk) && FW_SAME(tperiod) && FW_SAME(dep_wk) && FW_SAME(xc_wk) &&
           FW_SAME(yc_wk) && FW_SAME(theta_wk) && FW_SAME(delta_wk) && FW_SAME(time_ramp) && FW_SAME(ywidth_wk) &&
           FW_SAME(freq_peak) && FW_SAME(freq_min) && FW_SAME(freq_max) && FW_SAME(gamma_tma) && FW_SAME(hmo) &&
           FW_SAME(theta_peak) && FW_SAME(sigma_theta) && FW_SAME(nfreq) && FW_SAME(ntheta) && FW_SAME(spreading) &&
           FW_SAME(spread_s) && FW_SAME(precision) && FW_SAME(track_hmax) && FW_SAME(track_hmin) &&
           FW_SAME(track_umax) && FW_SAME(track_mfmax) && FW_SAME(steady_time) && FW_SAME(t_intv_mean) &&
           FW_SAME(track_roller) && FW_SAME(track_radiation);
#undef FW_SAME
}

// the Grid values fw_init (and fw_set_scalar "T_brk") set, taken from src
void copy_init_grid(Grid &dst, const Grid &src) {
    dst.T_brk = src.T_brk;
    dst.width_wk = src.width_wk;
    dst.D_gen = src.D_gen;
    dst.beta_gen = src.beta_gen;
    dst.rlamda = src.rlamda;
    dst.ilo = src.ilo;
    dst.ihi = src.ihi;
    dst.jlo = src.jlo;
    dst.jhi = src.jhi;
    fill_float_constants(dst);
}

template <typename T> void ck_offsets(fw_ctx *c, CkHeader &h, void **band) {
    fw::Fields<T> &f = c->F<T>();
    const char *a = (const char *)c->arena;
    h.off_mask = (const char *)f.MASK - a;
    h.off_maskn = (const char *)f.MASKn - a;
    h.off_age = (const char *)f.AGE - a;
    h.off_agen = (const char *)f.AGEn - a;
    band[0] = f.Cm;
    band[1] = f.Sm;
}

template <typename T> void ck_set_offsets(fw_ctx *c, const CkHeader &h) {
    fw::Fields<T> &f = c->F<T>();
    char *a = (char *)c->arena;
    f.MASK = (uint8_t *)(a + h.off_mask);
    f.MASKn = (uint8_t *)(a + h.off_maskn);
    f.AGE = (T *)(a + h.off_age);
    f.AGEn = (T *)(a + h.off_agen);
}

size_t band_bytes(const fw_ctx *c, const Grid &g) {
    if (c->p.wavemaker != FW_WK_JON_2D || g.ihi < g.ilo || g.jhi < g.jlo) return 0;
    const size_t es = c->p.precision == FW_PREC_FP64 ? sizeof(double) : sizeof(float);
    return (size_t)(g.ihi - g.ilo + 1) * (size_t)(g.jhi - g.jlo + 1) * (size_t)c->p.nfreq * es;
}

// device <-> file through one pinned host buffer, in pieces
const size_t kCkChunk = 64u << 20;

int ck_write(fw_ctx *c, FILE *fp, const void *dev, size_t n, void *pin) {
    for (size_t o = 0; o < n; o += kCkChunk) {
        const size_t k = std::min(kCkChunk, n - o);
        cudaError_t e = cudaMemcpyAsync(pin, (const char *)dev + o, k, cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) return cuda_status(c, e);
        if (std::fwrite(pin, 1, k, fp) != k) return FW_ERR_IO;
    }
    return FW_OK;
}

int ck_read(fw_ctx *c, FILE *fp, void *dev, size_t n, void *pin) {
    for (size_t o = 0; o < n; o += kCkChunk) {
        const size_t k = std::min(kCkChunk, n - o);
        if (std::fread(pin, 1, k, fp) != k) return FW_ERR_IO;
        cudaError_t e = cudaMemcpyAsync((char *)dev + o, pin, k, cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) return cuda_status(c, e);
    }
    return FW_OK;
}

struct PinnedBuf {
    void *p = nullptr;
    explicit PinnedBuf(size_t n) {
        if (cudaMallocHost(&p, n) != cudaSuccess) {
            cudaGetLastError();
            p = nullptr;
        }
    }
    ~PinnedBuf() {
        if (p) cudaFreeHost(p);
    }
};

struct FileCloser {
    FILE *f;
    ~FileCloser() {
        if (f) std::fclose(f);
    }
};

}  // namespace
extern "C" {

int fw_checkpoint(fw_ctx *c, const char *path) {
    if (!path) return FW_ERR_BAD_PARAM;
    int rc = check_ready(c);
    if (rc != FW_OK) return rc;
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_status(c, e);
    CkHeader h;
    std::memset(&h, 0, sizeof(h));
    std::memcpy(h.magic, kCkMagic, sizeof(h.magic));
    h.sizeof_params = (uint32_t)sizeof(fw_params);
    h.sizeof_grid = (uint32_t)sizeof(Grid);
    h.precision = c->p.precision;
    h.arena_bytes = c->arena_bytes;
    h.band_bytes = band_bytes(c, c->g);
    h.EtaBlowVal = c->EtaBlowVal;
    void *band[2];
    if (c->p.precision == FW_PREC_FP64) ck_offsets<double>(c, h, band);
    else ck_offsets<float>(c, h, band);
    if (h.band_bytes && (!band[0] || !band[1])) return FW_ERR_NOT_READY;
    PinnedBuf pin(std::min(kCkChunk, std::max(h.arena_bytes, (uint64_t)1)));
    if (!pin.p) return FW_ERR_OOM;
    FileCloser fc{std::fopen(path, "wb")};
    if (!fc.f) return FW_ERR_IO;
    if (std::fwrite(&h, sizeof(h), 1, fc.f) != 1 || std::fwrite(&c->p, sizeof(fw_params), 1, fc.f) != 1 ||
        std::fwrite(&c->g, sizeof(Grid), 1, fc.f) != 1)
        return FW_ERR_IO;
    if ((rc = ck_write(c, fc.f, c->arena, c->arena_bytes, pin.p)) != FW_OK) return rc;
    for (int k = 0; k < 2 && h.band_bytes; k++)
        if ((rc = ck_write(c, fc.f, band[k], h.band_bytes, pin.p)) != FW_OK) return rc;
    if (std::fflush(fc.f) != 0) return FW_ERR_IO;
    std::FILE *f = fc.f;
    fc.f = nullptr;
    return std::fclose(f) == 0 ? FW_OK : FW_ERR_IO;
}

int fw_restore(fw_ctx *c, const char *path) {
    if (!c || !path) return FW_ERR_BAD_PARAM;
    if (c->sticky_error) return FW_ERR_CUDA;
    FileCloser fc{std::fopen(path, "rb")};
    if (!fc.f) return FW_ERR_IO;
    CkHeader h;
    fw_params p;
    Grid g;
    if (std::fread(&h, sizeof(h), 1, fc.f) != 1 || std::memcmp(h.magic, kCkMagic, sizeof(h.magic)) != 0 ||
        h.sizeof_params != sizeof(fw_params) || h.sizeof_grid != sizeof(Grid) ||
        std::fread(&p, sizeof(p), 1, fc.f) != 1 || std::fread(&g, sizeof(g), 1, fc.f) != 1)
        return FW_ERR_IO;
    // the saved run must be one this context could have run: the same
    // parameters, the same arena, and a Grid that differs from this one's
    // only in what fw_init sets
    if (!same_params(p, c->p) || h.arena_bytes != c->arena_bytes) return FW_ERR_BAD_PARAM;
    Grid want = c->g;
    copy_init_grid(want, g);
    if (std::memcmp(&want, &g, sizeof(Grid)) != 0) return FW_ERR_BAD_PARAM;
    if (h.band_bytes != band_bytes(c, g)) return FW_ERR_IO;
    // the ping-pong buffers must be the two this context carved
    const bool fp64 = c->p.precision == FW_PREC_FP64;
    CkHeader mine;
    void *band[2];
    if (fp64) ck_offsets<double>(c, mine, band);
    else ck_offsets<float>(c, mine, band);
    const bool mask_ok = (h.off_mask == mine.off_mask && h.off_maskn == mine.off_maskn) ||
                         (h.off_mask == mine.off_maskn && h.off_maskn == mine.off_mask);
    const bool age_ok = (h.off_age == mine.off_age && h.off_agen == mine.off_agen) ||
                        (h.off_age == mine.off_agen && h.off_agen == mine.off_age);
    if (!mask_ok || !age_ok) return FW_ERR_IO;
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_status(c, e);
    // band tables: (re)allocate to the saved size
    void *nb[2] = {nullptr, nullptr};
    if (h.band_bytes) {
        if (cudaMalloc(&nb[0], h.band_bytes) != cudaSuccess || cudaMalloc(&nb[1], h.band_bytes) != cudaSuccess) {
            cudaGetLastError();
            if (nb[0]) cudaFree(nb[0]);
            return FW_ERR_OOM;
        }
    }
    PinnedBuf pin(std::min(kCkChunk, std::max(h.arena_bytes, (uint64_t)1)));
    int rc = pin.p ? FW_OK : FW_ERR_OOM;
    // from here a failure leaves the context un-initialised: its arena may
    // hold part of the file
    c->initialized = 0;
    if (rc == FW_OK) rc = ck_read(c, fc.f, c->arena, c->arena_bytes, pin.p);
    for (int k = 0; k < 2 && h.band_bytes && rc == FW_OK; k++) rc = ck_read(c, fc.f, nb[k], h.band_bytes, pin.p);
    if (rc == FW_OK && std::fgetc(fc.f) != EOF) rc = FW_ERR_IO;  // trailing bytes: not this format
    if (rc != FW_OK) {
        for (void *b : nb)
            if (b) cudaFree(b);
        return rc;
    }
    for (void *b : band)
        if (b) cudaFree(b);
    if (fp64) {
        ck_set_offsets<double>(c, h);
        c->fd.Cm = (double *)nb[0];
        c->fd.Sm = (double *)nb[1];
    } else {
        ck_set_offsets<float>(c, h);
        c->ff.Cm = (float *)nb[0];
        c->ff.Sm = (float *)nb[1];
    }
    c->g = g;
    c->EtaBlowVal = h.EtaBlowVal;
    if (c->graph) {
        cudaGraphExecDestroy(c->graph);
        c->graph = nullptr;
    }
    c->invalidate_graphs();
    c->initialized = 1;
    return FW_OK;
}

// ---------------------------------------------------------------------------
// Asynchronous output: PREVIEW's field transfers (io.F:4304-4621) without
// holding the step.  The snapshot is taken on the step stream, so it sees
// the state after every step enqueued before it; the device-to-host copies
// run on a second stream while later steps run.
// ---------------------------------------------------------------------------
// both output streams and events, created on first use
static int ensure_out_stream(fw_ctx *c) {
    if (c->out_stream) return FW_OK;
    cudaError_t e = cudaStreamCreateWithFlags(&c->out_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->out_ready, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->out_done, cudaEventDisableTiming);
    return cuda_status(c, e);
}

int fw_output_wait(fw_ctx *c) {
    if (!c) return FW_ERR_BAD_PARAM;
    if (!c->out_pending) return FW_OK;
    cudaError_t e = cudaEventSynchronize(c->out_done);
    c->out_pending = 0;
    return cuda_status(c, e);
}

int fw_output_done(fw_ctx *c) {
    if (!c) return FW_ERR_BAD_PARAM;
    if (!c->out_pending) return 1;
    cudaError_t e = cudaEventQuery(c->out_done);
    if (e == cudaErrorNotReady) return 0;
    if (e != cudaSuccess) return cuda_status(c, e);
    c->out_pending = 0;
    return 1;
}

int fw_output_begin(fw_ctx *c, int n, const char *const *names, void *const *host) {
    int rc = check_ready(c);
    if (rc != FW_OK) return rc;
    if (n < 1 || !names || !host) return FW_ERR_BAD_PARAM;
    const bool fp64 = c->p.precision == FW_PREC_FP64;
    std::vector<FieldRef> refs((size_t)n);
    std::vector<size_t> off((size_t)n + 1, 0);
    for (int k = 0; k < n; k++) {
        if (!names[k] || !host[k]) return FW_ERR_BAD_PARAM;
        const bool ok = fp64 ? find_field<double>(c, names[k], refs[k]) : find_field<float>(c, names[k], refs[k]);
        if (!ok) return FW_ERR_BAD_PARAM;
        int w, h;
        extent(c, refs[k].kind, w, h);
        const size_t bytes = (size_t)w * h * (refs[k].is_mask ? sizeof(int) : sizeof(double));
        off[k + 1] = off[k] + (bytes + 255) / 256 * 256;
    }
    // the previous snapshot's copies read out_buf: let them finish
    if ((rc = fw_output_wait(c)) != FW_OK) return rc;
    cudaError_t e = cudaSuccess;
    if ((rc = ensure_out_stream(c)) != FW_OK) return rc;
    if (off[n] > c->out_cap) {
        // nothing reads the old buffer: the copies waited for above ran
        // after the previous snapshot's kernels
        if (c->out_buf) cudaFree(c->out_buf);
        c->out_buf = nullptr;
        c->out_cap = 0;
        if (cudaMalloc(&c->out_buf, off[n]) != cudaSuccess) {
            cudaGetLastError();
            return FW_ERR_OOM;
        }
        c->out_cap = off[n];
    }
    char *buf = (char *)c->out_buf;
    for (int k = 0; k < n && e == cudaSuccess; k++) {
        const FieldRef &r = refs[k];
        int w, h;
        extent(c, r.kind, w, h);
        if (!r.is_mask && fp64)
            e = cudaMemcpy2DAsync(buf + off[k], (size_t)w * sizeof(double), r.ptr, (size_t)c->g.pitch * sizeof(double),
                                  (size_t)w * sizeof(double), (size_t)h, cudaMemcpyDeviceToDevice, c->stream);
        else
            convert_out(c, r.ptr, r.is_mask, buf + off[k], w, h);
    }
    if (e == cudaSuccess) e = cudaEventRecord(c->out_ready, c->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(c->out_stream, c->out_ready, 0);
    for (int k = 0; k < n && e == cudaSuccess; k++) {
        int w, h;
        extent(c, refs[k].kind, w, h);
        const size_t bytes = (size_t)w * h * (refs[k].is_mask ? sizeof(int) : sizeof(double));
        e = cudaMemcpyAsync(host[k], buf + off[k], bytes, cudaMemcpyDeviceToHost, c->out_stream);
    }
    if (e == cudaSuccess) e = cudaEventRecord(c->out_done, c->out_stream);
    if (e != cudaSuccess) return cuda_status(c, e);
    c->out_pending = 1;
    return finish(c);
}

// Several fields from the host at once: every plane is copied into a device
// input buffer on the second stream, and each conversion into its field
// starts on the step stream as soon as that plane has arrived, so copies and
// conversions overlap; one wait at the end.
int fw_set_fields(fw_ctx *c, int n, const char *const *names, const void *const *host) {
    if (!c) return FW_ERR_BAD_PARAM;
    if (c->sticky_error) return FW_ERR_CUDA;
    if (n < 1 || n > 16 || !names || !host) return FW_ERR_BAD_PARAM;
    const bool fp64 = c->p.precision == FW_PREC_FP64;
    std::vector<FieldRef> refs((size_t)n);
    std::vector<size_t> off((size_t)n + 1, 0);
    for (int k = 0; k < n; k++) {
        if (!names[k] || !host[k]) return FW_ERR_BAD_PARAM;
        const bool ok = fp64 ? find_field<double>(c, names[k], refs[k]) : find_field<float>(c, names[k], refs[k]);
        if (!ok) return FW_ERR_BAD_PARAM;
        int w, h;
        extent(c, refs[k].kind, w, h);
        const size_t bytes = (size_t)w * h * (refs[k].is_mask ? sizeof(int) : sizeof(double));
        off[k + 1] = off[k] + (bytes + 255) / 256 * 256;
    }
    int rc = ensure_out_stream(c);
    if (rc != FW_OK) return rc;
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < n && e == cudaSuccess; k++)
        if (!c->in_ev[k]) e = cudaEventCreateWithFlags(&c->in_ev[k], cudaEventDisableTiming);
    if (e != cudaSuccess) return cuda_status(c, e);
    // the step stream may still read the buffer (an earlier call's
    // conversions): it is idle after this wait
    if ((e = cudaStreamSynchronize(c->stream)) != cudaSuccess) return cuda_status(c, e);
    if (off[n] > c->in_cap) {
        if (c->in_buf) cudaFree(c->in_buf);
        c->in_buf = nullptr;
        c->in_cap = 0;
        if (cudaMalloc(&c->in_buf, off[n]) != cudaSuccess) {
            cudaGetLastError();
            return FW_ERR_OOM;
        }
        c->in_cap = off[n];
    }
    char *buf = (char *)c->in_buf;
    // the second stream must not start before the step stream's earlier work
    e = cudaEventRecord(c->out_ready, c->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(c->out_stream, c->out_ready, 0);
    for (int k = 0; k < n && e == cudaSuccess; k++) {
        const FieldRef &r = refs[k];
        int w, h;
        extent(c, r.kind, w, h);
        const size_t bytes = (size_t)w * h * (r.is_mask ? sizeof(int) : sizeof(double));
        e = cudaMemcpyAsync(buf + off[k], host[k], bytes, cudaMemcpyHostToDevice, c->out_stream);
        if (e == cudaSuccess) e = cudaEventRecord(c->in_ev[k], c->out_stream);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(c->stream, c->in_ev[k], 0);
        if (e != cudaSuccess) break;
        if (!r.is_mask && fp64)
            e = cudaMemcpy2DAsync(r.ptr, (size_t)c->g.pitch * sizeof(double), buf + off[k], (size_t)w * sizeof(double),
                                  (size_t)w * sizeof(double), (size_t)h, cudaMemcpyDeviceToDevice, c->stream);
        else
            convert_in(c, buf + off[k], r.is_mask, r.ptr, w, h);
        // the mixed build's double Depth of the total-depth tests
        if (e == cudaSuccess && !fp64 && std::strcmp(names[k], "Depth") == 0)
            e = cudaMemcpy2DAsync(c->ff.DepthD, (size_t)c->g.pitch * sizeof(double), buf + off[k],
                                  (size_t)w * sizeof(double), (size_t)w * sizeof(double), (size_t)h,
                                  cudaMemcpyDeviceToDevice, c->stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_status(c, e);
    return finish(c);
}

// Several fields to the host at once: the asynchronous output's snapshot and
// copies, then the wait
int fw_get_fields(fw_ctx *c, int n, const char *const *names, void *const *host) {
    int rc = fw_output_begin(c, n, names, host);
    if (rc != FW_OK) return rc;
    return fw_output_wait(c);
}

// n fields to or from float host arrays at once.  The mixed build's fields
// are floats in the host layout apart from the pitch: each plane crosses
// the host link as one contiguous copy, on the second stream, into (or out
// of) the device input buffer, and a device-side 2-D copy on the step
// stream moves it to (or from) the pitched field, so the copies of one
// plane overlap the device copies of the next.  The FP64 build converts
// through the staging plane field by field (fw_get_field_f32 /
// fw_set_field_f32).
static int f32_planes(fw_ctx *c, int n, const char *const *names, std::vector<FieldRef> &refs,
                      std::vector<size_t> &off) {
    refs.assign((size_t)n, FieldRef{});
    off.assign((size_t)n + 1, 0);
    for (int k = 0; k < n; k++) {
        if (!names[k] || !find_field<float>(c, names[k], refs[k]) || refs[k].is_mask) return FW_ERR_BAD_PARAM;
        int w, h;
        extent(c, refs[k].kind, w, h);
        off[k + 1] = off[k] + ((size_t)w * h * sizeof(float) + 255) / 256 * 256;
    }
    int rc = ensure_out_stream(c);
    if (rc != FW_OK) return rc;
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < n && e == cudaSuccess; k++)
        if (!c->in_ev[k]) e = cudaEventCreateWithFlags(&c->in_ev[k], cudaEventDisableTiming);
    // the step stream may still use the buffer (an earlier call): it is
    // idle after this wait
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_status(c, e);
    if (off[n] > c->in_cap) {
        if (c->in_buf) cudaFree(c->in_buf);
        c->in_buf = nullptr;
        c->in_cap = 0;
        if (cudaMalloc(&c->in_buf, off[n]) != cudaSuccess) {
            cudaGetLastError();
            return FW_ERR_OOM;
        }
        c->in_cap = off[n];
    }
    return FW_OK;
}

// Float host arrays that the GPU can address (page-locked memory: the
// caller's fw_host_alloc or cudaHostAlloc buffers) are read and written in
// place by one kernel per call, whose loads and stores cross the host link
// from every SM at once, and which scatters to (or gathers from) the pitched
// fields itself: no copy engine, no staging plane.  Other host arrays take
// the copy path below.
struct HostPlanes {
    float *host[16];   // the host arrays, through their device addresses
    float *dev[16];    // the pitched fields
    double *devd[16];  // set in: the double copy of Depth of the total-depth tests, else null
    int w[16], h[16];
    int pitch;
};

static __global__ void k_host_in_f32(HostPlanes hp) {
    const int k = blockIdx.y, w = hp.w[k], h = hp.h[k];
    const float *src = hp.host[k];
    float *dst = hp.dev[k];
    double *dd = hp.devd[k];
    const long long n = (long long)w * h;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e % w), j = (int)(e / w);
        const float v = src[e];
        const size_t q = (size_t)i + (size_t)j * hp.pitch;
        dst[q] = v;
        if (dd) dd[q] = (double)v;
    }
}

static __global__ void k_host_out_f32(HostPlanes hp) {
    const int k = blockIdx.y, w = hp.w[k], h = hp.h[k];
    float *dst = hp.host[k];
    const float *src = hp.dev[k];
    const long long n = (long long)w * h;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e % w), j = (int)(e / w);
        dst[e] = src[(size_t)i + (size_t)j * hp.pitch];
    }
}

// the device addresses of n page-locked host arrays; false if any is not
static bool host_views(int n, const void *const *host, float **dev) {
    for (int k = 0; k < n; k++) {
        cudaPointerAttributes a;
        if (cudaPointerGetAttributes(&a, host[k]) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        if (a.type != cudaMemoryTypeHost || !a.devicePointer) return false;
        dev[k] = (float *)a.devicePointer;
    }
    return true;
}

// the mixed build's fields of n names for the direct path
static bool host_planes(fw_ctx *c, int n, const char *const *names, const void *const *host, bool in,
                        HostPlanes &hp) {
    if (!host_views(n, host, hp.host)) return false;
    for (int k = 0; k < n; k++) {
        FieldRef r;
        if (!names[k] || !find_field<float>(c, names[k], r) || r.is_mask) return false;
        hp.dev[k] = (float *)r.ptr;
        hp.devd[k] = in && std::strcmp(names[k], "Depth") == 0 ? c->ff.DepthD : nullptr;
        extent(c, r.kind, hp.w[k], hp.h[k]);
    }
    hp.pitch = c->g.pitch;
    return true;
}

static int host_planes_run(fw_ctx *c, int n, HostPlanes &hp, bool in) {
    int dev = 0, nsm = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return cuda_status(c, e);
    const dim3 grid((unsigned)std::max(1, 4 * nsm / n), (unsigned)n);
    if (in) k_host_in_f32<<<grid, 512, 0, c->stream>>>(hp);
    else k_host_out_f32<<<grid, 512, 0, c->stream>>>(hp);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_status(c, e);
    return in ? finish(c) : FW_OK;
}

int fw_set_fields_f32(fw_ctx *c, int n, const char *const *names, const float *const *host) {
    if (!c) return FW_ERR_BAD_PARAM;
    if (c->sticky_error) return FW_ERR_CUDA;
    if (n < 1 || n > 16 || !names || !host) return FW_ERR_BAD_PARAM;
    for (int k = 0; k < n; k++)
        if (!host[k]) return FW_ERR_BAD_PARAM;
    if (c->p.precision == FW_PREC_FP64) {
        for (int k = 0; k < n; k++) {
            const int rc = fw_set_field_f32(c, names[k], host[k]);
            if (rc != FW_OK) return rc;
        }
        return FW_OK;
    }
    HostPlanes hp;
    if (host_planes(c, n, names, (const void *const *)host, true, hp)) return host_planes_run(c, n, hp, true);
    std::vector<FieldRef> refs;
    std::vector<size_t> off;
    int rc = f32_planes(c, n, names, refs, off);
    if (rc != FW_OK) return rc;
    char *buf = (char *)c->in_buf;
    cudaError_t e = cudaEventRecord(c->out_ready, c->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(c->out_stream, c->out_ready, 0);
    for (int k = 0; k < n && e == cudaSuccess; k++) {
        int w, h;
        extent(c, refs[k].kind, w, h);
        e = cudaMemcpyAsync(buf + off[k], host[k], (size_t)w * h * sizeof(float), cudaMemcpyHostToDevice,
                            c->out_stream);
        if (e == cudaSuccess) e = cudaEventRecord(c->in_ev[k], c->out_stream);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(c->stream, c->in_ev[k], 0);
        if (e == cudaSuccess)
            e = cudaMemcpy2DAsync(refs[k].ptr, (size_t)c->g.pitch * sizeof(float), buf + off[k], (size_t)w * sizeof(float),
                                  (size_t)w * sizeof(float), (size_t)h, cudaMemcpyDeviceToDevice, c->stream);
        // the double Depth of the total-depth tests, widened from the floats
        if (e == cudaSuccess && std::strcmp(names[k], "Depth") == 0)
            convert_in_f32(c, (const float *)(buf + off[k]), c->ff.DepthD, w, h);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_status(c, e);
    return finish(c);
}

int fw_get_fields_f32(fw_ctx *c, int n, const char *const *names, float *const *host) {
    if (!c) return FW_ERR_BAD_PARAM;
    if (c->sticky_error) return FW_ERR_CUDA;
    if (n < 1 || n > 16 || !names || !host) return FW_ERR_BAD_PARAM;
    for (int k = 0; k < n; k++)
        if (!host[k]) return FW_ERR_BAD_PARAM;
    if (c->p.precision == FW_PREC_FP64) {
        for (int k = 0; k < n; k++) {
            const int rc = fw_get_field_f32(c, names[k], host[k]);
            if (rc != FW_OK) return rc;
        }
        return FW_OK;
    }
    HostPlanes hp;
    if (host_planes(c, n, names, (const void *const *)host, false, hp)) return host_planes_run(c, n, hp, false);
    std::vector<FieldRef> refs;
    std::vector<size_t> off;
    int rc = f32_planes(c, n, names, refs, off);
    if (rc != FW_OK) return rc;
    char *buf = (char *)c->in_buf;
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < n && e == cudaSuccess; k++) {
        int w, h;
        extent(c, refs[k].kind, w, h);
        e = cudaMemcpy2DAsync(buf + off[k], (size_t)w * sizeof(float), refs[k].ptr, (size_t)c->g.pitch * sizeof(float),
                              (size_t)w * sizeof(float), (size_t)h, cudaMemcpyDeviceToDevice, c->stream);
        if (e == cudaSuccess) e = cudaEventRecord(c->in_ev[k], c->stream);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(c->out_stream, c->in_ev[k], 0);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(host[k], buf + off[k], (size_t)w * h * sizeof(float), cudaMemcpyDeviceToHost,
                                c->out_stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->out_stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    return cuda_status(c, e);
}

int fw_host_alloc(size_t bytes, void **ptr) {
    if (!ptr) return FW_ERR_BAD_PARAM;
    *ptr = nullptr;
    if (cudaMallocHost(ptr, bytes) != cudaSuccess) {
        cudaGetLastError();
        *ptr = nullptr;
        return FW_ERR_OOM;
    }
    return FW_OK;
}

int fw_host_free(void *ptr) {
    if (ptr && cudaFreeHost(ptr) != cudaSuccess) {
        cudaGetLastError();
        return FW_ERR_CUDA;
    }
    return FW_OK;
}

long long fw_launch_count(fw_ctx *c) { return c ? c->launches : -1; }

int fw_time_kernel(fw_ctx *c, const char *name, int nrep, double *ms_per_launch) {
    int rc = check_ready(c);
    if (rc != FW_OK) return rc;
    if (!name || nrep < 1 || !ms_per_launch) return FW_ERR_BAD_PARAM;
    cudaEvent_t a, b;
    if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) return cuda_status(c, cudaGetLastError());
    const bool fp64 = c->p.precision == FW_PREC_FP64;
    // one untimed launch validates the name and warms the caches
    if ((fp64 ? launch_by_name<double>(c, name) : launch_by_name<float>(c, name)) != 0) {
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        return FW_ERR_BAD_PARAM;
    }
    cudaError_t e = cudaEventRecord(a, c->stream);
    for (int k = 0; k < nrep && e == cudaSuccess; k++) {
        if (fp64) launch_by_name<double>(c, name);
        else launch_by_name<float>(c, name);
    }
    if (e == cudaSuccess) e = cudaEventRecord(b, c->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(b);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (e != cudaSuccess) return cuda_status(c, e);
    *ms_per_launch = (double)ms / nrep;
    return finish(c);
}
void *fw_stream(fw_ctx *c) { return c ? (void *)c->stream : nullptr; }

int fw_get_tuning(fw_ctx *c, int *t) {
    if (!c || !t) return FW_ERR_BAD_PARAM;
    std::memcpy(t, c->tune, sizeof(c->tune));
    return FW_OK;
}

int fw_set_tuning(fw_ctx *c, const int *t) {
    if (!c || !t) return FW_ERR_BAD_PARAM;
    if (!tune_valid(c, t)) return FW_ERR_BAD_PARAM;
    std::memcpy(c->tune, t, sizeof(c->tune));
    c->invalidate_graphs();
    return FW_OK;
}

int fw_autotune(fw_ctx *c, int flags) {
    int rc = check_ready(c);
    if (rc != FW_OK) return rc;
    // size class: the number of bits of Mglob - 1 and Nglob - 1 (grids
    // within one power of two share a tuning), plus the kernels' path
    auto bits = [](int v) {
        int b = 0;
        for (unsigned u = (unsigned)(v - 1); u; u >>= 1) b++;
        return b;
    };
    const std::array<long long, 8> key = {c->p.precision, bits(c->g.Mglob), bits(c->g.Nglob), c->g.dispersion,
                                          c->g.show_breaking, c->g.periodic, c->factored, c->g.direct_sponge};
    if (!(flags & FW_TUNE_FRESH)) {
        std::lock_guard<std::mutex> lk(tune_mu);
        auto it = tune_cache.find(key);
        if (it != tune_cache.end()) {
            std::memcpy(c->tune, it->second.data(), sizeof(c->tune));
            c->invalidate_graphs();
            return FW_OK;
        }
    }
    // the candidates run on the real state; save it and put it back after
    void *save = nullptr;
    if (cudaMalloc(&save, c->arena_bytes) != cudaSuccess) {
        cudaGetLastError();
        return FW_ERR_OOM;
    }
    cudaError_t e = cudaMemcpyAsync(save, c->arena, c->arena_bytes, cudaMemcpyDeviceToDevice, c->stream);
    const bool fp64 = c->p.precision == FW_PREC_FP64;
    const bool disp = c->g.dispersion != 0, pmb = disp && c->g.show_breaking;
    const bool on_path[fw::TK_N] = {disp, disp, true, pmb, true};
    for (int sweep = 0; sweep < 2 && e == cudaSuccess; sweep++) {
        for (int k = 0; k < fw::TK_N && e == cudaSuccess; k++) {
            if (!on_path[k]) continue;
            double best = 1e30;
            int bx = c->tune[2 * k], by = c->tune[2 * k + 1];
            for (const auto &cand : CELL_CANDIDATES) {
                c->tune[2 * k] = cand[0];
                c->tune[2 * k + 1] = cand[1];
                const double ms = time_named(c, fp64, TUNE_NAMES[k], e);
                if (ms < best) {
                    best = ms;
                    bx = cand[0];
                    by = cand[1];
                }
            }
            c->tune[2 * k] = bx;
            c->tune[2 * k + 1] = by;
        }
        for (int dir = 0; dir < 2 && e == cudaSuccess; dir++) {
            double best = 1e30;
            int pick = c->tune[fw::TUNE_FLUX + dir], pick_tma = c->tune[fw::TUNE_FLUX_TMA + dir];
            for (int tma = 0; tma < 2; tma++)
                for (int fy : {8, 16, 32}) {
                    c->tune[fw::TUNE_FLUX + dir] = fy;
                    c->tune[fw::TUNE_FLUX_TMA + dir] = tma;
                    if (!tune_valid(c, c->tune)) continue;
                    const double ms = time_named(c, fp64, dir == 0 ? "flux_x" : "flux_y", e);
                    if (ms < best) {
                        best = ms;
                        pick = fy;
                        pick_tma = tma;
                    }
                }
            c->tune[fw::TUNE_FLUX + dir] = pick;
            c->tune[fw::TUNE_FLUX_TMA + dir] = pick_tma;
        }
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(c->arena, save, c->arena_bytes, cudaMemcpyDeviceToDevice, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cudaFree(save);
    c->invalidate_graphs();
    if (e != cudaSuccess) return cuda_status(c, e);
    {
        std::lock_guard<std::mutex> lk(tune_mu);
        std::array<int, FW_TUNE_LEN> v;
        std::memcpy(v.data(), c->tune, sizeof(c->tune));
        tune_cache[key] = v;
    }
    return finish(c);
}

}  // extern "C"
