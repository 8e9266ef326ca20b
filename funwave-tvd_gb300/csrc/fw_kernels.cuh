// fw_kernels.cu -- sm_103a kernels of the FUNWAVE-TVD SSP-RK3 stage.
//
// Every kernel reproduces one or more of the reference's Fortran units on
// the device-resident state (layout in fw_internal.h).  Index ranges,
// in-place update orders and stale-value semantics follow the reference:
//   - ghost cells hold exactly what EXCHANGE / EXCHANGE_DISPERSION leave
//     (PHI_COLL order: periodic copy, x mirror on interior rows, y mirror on
//     all columns; bc.F:631-1272), including the periodic corner cells that
//     keep the value of the x-ghost cell they copy from before that cell is
//     refilled;
//   - BOUNDARY_CONDITION's overlapping dry-face writes (bc.F:214-293) are
//     resolved per face by the write that comes last in the reference's loop;
//   - UPDATE_MASK is a Jacobi update (masks.F:75-143) with the order-
//     dependent Depthx/Depthy reset (masks.F:152-161) resolved per face;
//   - the breaking AGE sweep (breaker.F:149-229) is an in-place Gauss-Seidel
//     sweep; it is reproduced exactly by evaluating every cell whose result
//     does not depend on its neighbours in parallel, then iterating the rest
//     (cells with AGE = 0 and Cbrk2 <= ETAt < Cbrk1) to the fixed point of
//     the sweep's acyclic dependency graph.
// T is the storage and arithmetic type of the bulk fields (double or
// float); the tridiagonal u/v recovery always runs in double.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <algorithm>
#include <cstring>

#include "fw_internal.h"
#include "fw_tc.cuh"

namespace fw {

#define IDX(i, j) ((size_t)(i) + (size_t)(j) * (size_t)g.pitch)

// pi as the reference stores it: a default-REAL literal (mod_param.F:71)
constexpr double PI_SP = (double)(float)3.141592653;
// the default-REAL literal 4.004 of SigWaveHeight (mixing.F:244)
constexpr double C4004_SP = (double)(float)4.004;
constexpr double GRAV = 9.81;
constexpr double SMALL = 0.000001;
constexpr double LARGE = 999999.0;

// bring the cache line of p into L1 (no value, no register): later loads of
// inputs that the compiler may not move above earlier stores then hit L1
__device__ __forceinline__ void prefetch_l1(const void *p) {
    asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
}
// a load of an array that the kernel does not write: the read-only data
// path, which also frees the compiler to issue it before the kernel's
// stores (the Fields pointers could otherwise alias them)
template <typename X> __device__ __forceinline__ X ro(const X *p) { return __ldg(p); }

__device__ __forceinline__ double fsqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float fsqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double fabs_(double x) { return fabs(x); }
__device__ __forceinline__ float fabs_(float x) { return fabsf(x); }
__device__ __forceinline__ double fcopysign(double a, double b) { return copysign(a, b); }
__device__ __forceinline__ float fcopysign(float a, float b) { return copysignf(a, b); }
__device__ __forceinline__ double fexp(double x) { return exp(x); }
__device__ __forceinline__ float fexp(float x) { return expf(x); }
__device__ __forceinline__ double fsin(double x) { return sin(x); }
__device__ __forceinline__ float fsin(float x) { return sinf(x); }
__device__ __forceinline__ double fcos(double x) { return cos(x); }
__device__ __forceinline__ float fcos(float x) { return cosf(x); }
__device__ __forceinline__ double ftanh(double x) { return tanh(x); }
__device__ __forceinline__ float ftanh(float x) { return tanhf(x); }
__device__ __forceinline__ double fatan2(double y, double x) { return atan2(y, x); }
__device__ __forceinline__ float fatan2(float y, float x) { return atan2f(y, x); }

// a constant of the grid block in the kernel's precision: the double member
// in FP64, its float copy f_<name> in the mixed path (no FP64 work there)
#define GC(name) (sizeof(T) == sizeof(double) ? (T)g.name : (T)g.f_##name)
// DT of the current step in the kernel's precision
#define DTV (sizeof(T) == sizeof(double) ? (T)f.dsc[S_DT] : (T)f.fsc[FS_DT])

// a 0/1 mask byte as a real, by a select instead of an integer-to-float
// conversion instruction
template <typename T> __device__ __forceinline__ T m2r(int m) { return m ? (T)1 : (T)0; }
// a small integer (|k| < 2^22) as a real; in float exactly, by placing k in
// the mantissa of 1.5*2^23 and subtracting that constant
template <typename T> __device__ __forceinline__ T i2r(int k) {
    if constexpr (sizeof(T) == sizeof(double)) return (T)k;
    else return __int_as_float(0x4B400000 + k) - 12582912.0f;
}
template <typename T> __device__ __forceinline__ T tmax(T a, T b) { return a > b ? a : b; }
template <typename T> __device__ __forceinline__ T tmin(T a, T b) { return a < b ? a : b; }

// ---------------------------------------------------------------------------
// exchange source of a ghost cell (PHI_COLL, serial branches)
// ---------------------------------------------------------------------------
__device__ __forceinline__ int mirror_x(const Grid &g, int i) {
    return i < g.ib ? 2 * g.ib - 1 - i : (i > g.ie ? 2 * g.ie + 1 - i : i);
}
__device__ __forceinline__ int mirror_y(const Grid &g, int j) {
    return j < g.jb ? 2 * g.jb - 1 - j : (j > g.je ? 2 * g.je + 1 - j : j);
}
// periodic-y source row of a ghost row (bc.F:735-740)
__device__ __forceinline__ int period_y(const Grid &g, int j) {
    return j < g.jb ? j + g.je - 2 : (j > g.je ? j - g.je + 2 : j);
}

// ---------------------------------------------------------------------------
// CAL_DISPERSION, part 1 (dispersion.F:62-289): masked derivatives at the
// exchange source of every cell, combined into the four sums the rest of
// the unit uses, plus ETAx/ETAy (exchanged) and ETAT.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(256) k_disp_a(Grid g, Fields<T> f) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= g.Mloc || j >= g.Nloc) return;
    const T DX = GC(DX), DY = GC(DY), mdf = GC(min_depth_frc);
    const size_t id = IDX(i, j);
    // ETAT from the previous stage's face fluxes (dispersion.F:103-119)
    if (i <= g.Mloc - 2 && j <= g.Nloc - 2) {
        if constexpr (sizeof(T) == sizeof(double))
            f.ETAT[id] = -(ro(f.P + (IDX(i + 1, j))) - ro(f.P + (id))) / DX - (ro(f.Q + (IDX(i, j + 1))) - ro(f.Q + (id))) / DY;
        else
            f.ETAT[id] = -(ro(f.P + (IDX(i + 1, j))) - ro(f.P + (id))) * GC(rdx) - (ro(f.Q + (IDX(i, j + 1))) - ro(f.Q + (id))) * GC(rdy);
    }

    const bool gx = (i < g.ib) || (i > g.ie);
    const bool gy = (j < g.jb) || (j > g.je);
    const int si = mirror_x(g, i);
    int sj = j;
    T sy3 = (T)1;  // sign of VTYPE 3 fields in a y ghost
    bool stale = false;
    if (gy) {
        if (g.periodic) {
            sj = period_y(g, j);
            stale = gx;  // periodic corner: keeps the pre-exchange value
        } else {
            sj = mirror_y(g, j);
            sy3 = (T)-1;
        }
    }
    const T sx2 = gx ? (T)-1 : (T)1;  // sign of VTYPE 2 fields in an x ghost

    const T m9 = m2r<T>(ro(f.MASK9 + (IDX(si, sj))));
    const bool wall = (si == g.ib) || (si == g.ie) || (sj == g.jb) || (sj == g.je);
#define LU(a, b) ro(f.U + (IDX(si + (a), sj + (b))))
#define LV(a, b) ro(f.V + (IDX(si + (a), sj + (b))))
#define LDU(a, b) (tmax(ro(f.Depth + (IDX(si + (a), sj + (b)))), mdf) * LU(a, b))
#define LDV(a, b) (tmax(ro(f.Depth + (IDX(si + (a), sj + (b)))), mdf) * LV(a, b))
    // FP64: the reference's divisions; mixed: reciprocal constants
    constexpr bool EXACT = sizeof(T) == sizeof(double);
    const T rdx2 = (T)g.f_rdx2, rdy2 = (T)g.f_rdy2, rdxy4 = (T)g.f_rdxy4;
#define DXX(F) (EXACT ? (((F(1, 0) - (T)2 * F(0, 0) + F(-1, 0)) / DX / DX) * m9) \
                      : ((F(1, 0) - (T)2 * F(0, 0) + F(-1, 0)) * rdx2 * m9))
#define DYY(F) (EXACT ? (((F(0, 1) - (T)2 * F(0, 0) + F(0, -1)) / DY / DY) * m9) \
                      : ((F(0, 1) - (T)2 * F(0, 0) + F(0, -1)) * rdy2 * m9))
#define DXY(F)                                                                                      \
    (wall ? (T)0                                                                                    \
          : (EXACT ? ((((F(1, 1) - F(1, -1)) / (T)2 / DY) - ((F(-1, 1) - F(-1, -1)) / (T)2 / DY)) / \
                      (T)2 / DX) * m9                                                               \
                   : (((F(1, 1) - F(1, -1)) - (F(-1, 1) - F(-1, -1))) * rdxy4 * m9)))
    const T Uxx = DXX(LU), Vyy = DYY(LV), Uxy = DXY(LU), Vxy = DXY(LV);
    const T DUxx = DXX(LDU), DVyy = DYY(LDV), DUxy = DXY(LDU), DVxy = DXY(LDV);
#undef LU
#undef LV
#undef LDU
#undef LDV
#undef DXX
#undef DYY
#undef DXY
    if constexpr (sizeof(T) == sizeof(double)) {
        // FP64: keep every exchanged term (VTYPE 2: Uxx DUxx; 3: Vyy DVyy;
        // 1: the cross derivatives), as EXCHANGE_DISPERSION leaves them
        f.Uxx[id] = sx2 * Uxx;
        f.DUxx[id] = sx2 * DUxx;
        f.Vyy[id] = sy3 * Vyy;
        f.DVyy[id] = sy3 * DVyy;
        f.Uxy[id] = Uxy;
        f.Vxy[id] = Vxy;
        f.DUxy[id] = DUxy;
        f.DVxy[id] = DVxy;
    } else {
        f.A[id] = sx2 * Uxx + Vxy;
        f.B[id] = sx2 * DUxx + DVxy;
        f.C[id] = Uxy + sy3 * Vyy;
        f.E[id] = DUxy + sy3 * DVyy;
    }
    // ETAx, ETAy: computed on the interior and exchanged only when Gamma2 > 0
    // (bc.F:395-398); without Gamma2 the ghosts keep their old values
    const bool exch = g.has_g2 != 0;
    if (exch || (g.show_breaking && !gx && !gy)) {
        const T dex = ro(f.Eta + (IDX(si + 1, sj))) - ro(f.Eta + (IDX(si - 1, sj)));
        const T dey = ro(f.Eta + (IDX(si, sj + 1))) - ro(f.Eta + (IDX(si, sj - 1)));
        const T ex = EXACT ? dex / DX / (T)2 * m9 : dex * (T)g.f_hdx * m9;
        const T ey = EXACT ? dey / DY / (T)2 * m9 : dey * (T)g.f_hdy * m9;
        if (!stale) {
            if (exch && g.periodic && gx && !gy) {
                // the periodic copy (bc.F:735-740) runs before the x mirror:
                // a corner cell receives this x-ghost cell's previous value
                if (j >= g.je - 2) {
                    f.ETAx[IDX(i, j - (g.je - 2))] = f.ETAx[id];
                    f.ETAy[IDX(i, j - (g.je - 2))] = f.ETAy[id];
                }
                if (j <= g.jb + 2) {
                    f.ETAx[IDX(i, j + g.je - 2)] = f.ETAx[id];
                    f.ETAy[IDX(i, j + g.je - 2)] = f.ETAy[id];
                }
            }
            f.ETAx[id] = sx2 * ex;
            f.ETAy[id] = sy3 * ey;
        }
    }
}

// ---------------------------------------------------------------------------
// CAL_DISPERSION, part 2 (dispersion.F:293-503): U4, V4 on every cell;
// U1p, V1p and U1pp+U2+U3, V1pp+V2+V3 on the interior.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(256, sizeof(T) == sizeof(float) ? 4 : 1) k_disp_b(Grid g, Fields<T> f) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= g.Mloc || j >= g.Nloc) return;
    const size_t id = IDX(i, j);
    const T DX = GC(DX), DY = GC(DY), mdf = GC(min_depth_frc);
    const T B1 = GC(Beta_1), B2 = GC(Beta_2), g2 = GC(gamma2), b2 = GC(b2);
    const T one = (T)1, two = (T)2, half = (T)0.5;
    const T D = f.Depth[id], reta = f.Eta[id], m9 = m2r<T>(f.MASK9[id]);
    constexpr bool EXACT = sizeof(T) == sizeof(double);
    T a, b, c, e;
    if constexpr (EXACT) {
        a = f.Uxx[id] + f.Vxy[id];
        b = f.DUxx[id] + f.DVxy[id];
        c = f.Uxy[id] + f.Vyy[id];
        e = f.DUxy[id] + f.DVyy[id];
    } else {
        a = f.A[id];
        b = f.B[id];
        c = f.C[id];
        e = f.E[id];
    }
    T u4 = (one / (T)3 - B1 + half * B1 * B1) * D * D * a + (B1 - one / two) * D * b;
    T v4 = (one / (T)3 - B1 + half * B1 * B1) * D * D * c + (B1 - one / two) * D * e;
    if (g.has_g2) {
        const T ken1 = (one / (T)6 - B1 + B1 * B1) * D * reta * B2 +
                       (one / two * B1 * B1 - one / (T)6) * reta * reta * B2 * B2;
        const T ken2 = (B1 - one / two) * reta * B2;
        u4 = u4 + g2 * m9 * (ken1 * a + ken2 * b);
        v4 = v4 + g2 * m9 * (ken1 * c + ken2 * e);
    }
    f.U4[id] = u4;
    f.V4[id] = v4;
    if (i < g.ib || i > g.ie || j < g.jb || j > g.je) return;

    f.U1p[id] = half * (one - B1) * (one - B1) * D * D * a + (B1 - one) * D * b;
    f.V1p[id] = half * (one - B1) * (one - B1) * D * D * c + (B1 - one) * D * e;
    if (!g.has_g2) return;

    const T DT = DTV;
    const T rDT = (T)f.fsc[FS_RDT];
    const T hdx = (T)g.f_hdx, hdy = (T)g.f_hdy;
    const T rdx2 = (T)g.f_rdx2, rdy2 = (T)g.f_rdy2, rdxy4 = (T)g.f_rdxy4;
    const bool wall = (i == g.ib) || (i == g.ie) || (j == g.jb) || (j == g.je);
#define AT(F, a_, b_) f.F[IDX(i + (a_), j + (b_))]
    const T UxxVxy = a, UxyVyy = c, HUxxHVxy = b, HUxyHVyy = e;
    T UxxVxy_x, UxxVxy_y, UxyVyy_x, UxyVyy_y, HUxxHVxy_x, HUxxHVxy_y, HUxyHVyy_x, HUxyHVyy_y;
    if constexpr (EXACT) {
        // (F1(I+1)+F2(I+1)-F1(I-1)-F2(I-1))/2/DX, evaluated left to right
#define DIFF(F1, F2, a1, b1, a2, b2, H) \
    ((AT(F1, a1, b1) + AT(F2, a1, b1) - AT(F1, a2, b2) - AT(F2, a2, b2)) / two / H)
        UxxVxy_x = DIFF(Uxx, Vxy, 1, 0, -1, 0, DX);
        UxxVxy_y = DIFF(Uxx, Vxy, 0, 1, 0, -1, DY);
        UxyVyy_x = DIFF(Uxy, Vyy, 1, 0, -1, 0, DX);
        UxyVyy_y = DIFF(Uxy, Vyy, 0, 1, 0, -1, DY);
        HUxxHVxy_x = DIFF(DUxx, DVxy, 1, 0, -1, 0, DX);
        HUxxHVxy_y = DIFF(DUxx, DVxy, 0, 1, 0, -1, DY);
        HUxyHVyy_x = DIFF(DUxy, DVyy, 1, 0, -1, 0, DX);
        HUxyHVyy_y = DIFF(DUxy, DVyy, 0, 1, 0, -1, DY);
#undef DIFF
    } else {
        const T hx = (T)g.f_hdx, hy = (T)g.f_hdy;
        UxxVxy_x = (AT(A, 1, 0) - AT(A, -1, 0)) * hx;
        UxxVxy_y = (AT(A, 0, 1) - AT(A, 0, -1)) * hy;
        UxyVyy_x = (AT(C, 1, 0) - AT(C, -1, 0)) * hx;
        UxyVyy_y = (AT(C, 0, 1) - AT(C, 0, -1)) * hy;
        HUxxHVxy_x = (AT(B, 1, 0) - AT(B, -1, 0)) * hx;
        HUxxHVxy_y = (AT(B, 0, 1) - AT(B, 0, -1)) * hy;
        HUxyHVyy_x = (AT(E, 1, 0) - AT(E, -1, 0)) * hx;
        HUxyHVyy_y = (AT(E, 0, 1) - AT(E, 0, -1)) * hy;
    }
    const T rh = D;
    const T rhx = EXACT ? (AT(Depth, 1, 0) - AT(Depth, -1, 0)) / two / DX : (AT(Depth, 1, 0) - AT(Depth, -1, 0)) * hdx;
    const T rhy = EXACT ? (AT(Depth, 0, 1) - AT(Depth, 0, -1)) / two / DY : (AT(Depth, 0, 1) - AT(Depth, 0, -1)) * hdy;
    const T ETAx = f.ETAx[id], ETAy = f.ETAy[id], ETAT = f.ETAT[id];
    // first derivatives of U, V, DU, DV (derivatives.F:123-162)
#define FD1X(F) (EXACT ? ((F(1, 0) - F(-1, 0)) / DX / two) * m9 : ((F(1, 0) - F(-1, 0)) * hdx) * m9)
#define FD1Y(F) (EXACT ? ((F(0, 1) - F(0, -1)) / DY / two) * m9 : ((F(0, 1) - F(0, -1)) * hdy) * m9)
#define LU_(a_, b_) AT(U, a_, b_)
#define LV_(a_, b_) AT(V, a_, b_)
    const T Ux = FD1X(LU_);
    const T Vx = FD1X(LV_);
    const T Uy = FD1Y(LU_);
    const T Vy = FD1Y(LV_);
#undef LU_
#undef LV_
#define DUP(a_, b_) (tmax(AT(Depth, a_, b_), mdf) * AT(U, a_, b_))
#define DVP(a_, b_) (tmax(AT(Depth, a_, b_), mdf) * AT(V, a_, b_))
    const T DUx = FD1X(DUP);
    const T DVy = FD1Y(DVP);
    // time derivatives Ut=(U-U0)/DT (dispersion.F:133-141) and their
    // derivatives; the cross derivatives are zero on the wall rows
#define UT(a_, b_) (EXACT ? ((AT(U, a_, b_) - AT(U0, a_, b_)) / DT) : ((AT(U, a_, b_) - AT(U0, a_, b_)) * rDT))
#define VT(a_, b_) (EXACT ? ((AT(V, a_, b_) - AT(V0, a_, b_)) / DT) : ((AT(V, a_, b_) - AT(V0, a_, b_)) * rDT))
#define DUT(a_, b_) (tmax(AT(Depth, a_, b_), mdf) * UT(a_, b_))
#define DVT(a_, b_) (tmax(AT(Depth, a_, b_), mdf) * VT(a_, b_))
#define D1X(F) FD1X(F)
#define D1Y(F) FD1Y(F)
#define D2X(F) (EXACT ? (((F(1, 0) - two * F(0, 0) + F(-1, 0)) / DX / DX) * m9) \
                      : ((F(1, 0) - two * F(0, 0) + F(-1, 0)) * rdx2 * m9))
#define D2Y(F) (EXACT ? (((F(0, 1) - two * F(0, 0) + F(0, -1)) / DY / DY) * m9) \
                      : ((F(0, 1) - two * F(0, 0) + F(0, -1)) * rdy2 * m9))
#define D2XY(F)                                                                                          \
    (wall ? (T)0                                                                                         \
          : (EXACT ? ((((F(1, 1) - F(1, -1)) / two / DY) - ((F(-1, 1) - F(-1, -1)) / two / DY)) / two / DX) * m9 \
                   : (((F(1, 1) - F(1, -1)) - (F(-1, 1) - F(-1, -1))) * rdxy4 * m9)))
    const T Utx = D1X(UT), Vty = D1Y(VT);
    const T Utxx = D2X(UT), Vtyy = D2Y(VT);
    const T Utxy = D2XY(UT), Vtxy = D2XY(VT);
    const T DUtx = D1X(DUT), DVty = D1Y(DVT);
    const T DUtxx = D2X(DUT), DVtyy = D2Y(DVT);
    const T DUtxy = D2XY(DUT), DVtxy = D2XY(DVT);
#undef D1X
#undef D1Y
#undef D2X
#undef D2Y
#undef D2XY
#undef UT
#undef VT
#undef DUT
#undef DVT
#undef DUP
#undef DVP
#undef FD1X
#undef FD1Y
    const T Uc = f.U[id], Vc = f.V[id];
#undef AT
    T U1pp = -reta * B2 * ETAx * B2 * (Utx + Vty) - half * reta * reta * B2 * B2 * (Utxx + Vtxy) -
             ETAx * B2 * (DUtx + DVty) - reta * B2 * (DUtxx + DVtxy);
    T V1pp = -reta * B2 * ETAy * B2 * (Utx + Vty) - half * reta * reta * B2 * B2 * (Utxy + Vtyy) -
             ETAy * B2 * (DUtx + DVty) - reta * B2 * (DUtxy + DVtyy);
    T ken1 = B1 * (one - B1) * rh * ETAT * B2 - B1 * B1 * reta * B2 * ETAT * B2;
    T ken2 = B1 * (one - B1) * rh * reta * B2 - half * B1 * B1 * reta * reta * B2 * B2;
    T ken3 = B1 * ETAT * B2;
    T ken4 = B1 * reta * B2;
    U1pp = U1pp - ken1 * UxxVxy - ken2 * (Utxx + Vtxy) + ken3 * HUxxHVxy + ken4 * (DUtxx + DVtxy);
    V1pp = V1pp - ken1 * UxyVyy - ken2 * (Utxy + Vtyy) + ken3 * HUxyHVyy + ken4 * (DUtxy + DVtyy);

    ken1 = (B1 - one) * (rhx + ETAx) * B2;
    ken2 = (B1 - one) * (rh + reta) * B2;
    ken3 = ((one - B1) * (one - B1) * rh * rhx * B2 * B2 - B1 * (one - B1) * (rhx * reta * B2 + rh * ETAx * B2) +
            (B1 * B1 - one) * reta * ETAx * B2 * B2);
    ken4 = (half * (one - B1) * (one - B1) * rh * rh * B2 * B2 - B1 * (one - B1) * rh * reta * B2 +
            half * (B1 * B1 - one) * reta * reta * B2 * B2);
    const T ken5 = ((one - B1) * (one - B1) * rh * rhy * B2 * B2 -
                    B1 * (one - B1) * (rhy * reta * B2 + rh * ETAy * B2) + (B1 * B1 - one) * reta * ETAy * B2 * B2);
    const T U2 = ken1 * (Uc * HUxxHVxy + Vc * HUxyHVyy) +
                 ken2 * (Ux * HUxxHVxy + Uc * HUxxHVxy_x + Vx * HUxyHVyy + Vc * HUxyHVyy_x) +
                 ken3 * (Uc * UxxVxy + Vc * UxyVyy) + ken4 * (Ux * UxxVxy + Uc * UxxVxy_x + Vx * UxyVyy + Vc * UxyVyy_x) +
                 B2 * B2 * (DUx + DVy + reta * B2 * (Ux + Vy)) * (HUxxHVxy + ETAx * B2 * (Ux + Vy) + reta * B2 * UxxVxy);
    ken1 = (B1 - one) * (rhy + ETAy) * B2;
    const T V2 = ken1 * (Uc * HUxxHVxy + Vc * HUxyHVyy) +
                 ken2 * (Uy * HUxxHVxy + Uc * HUxxHVxy_y + Vy * HUxyHVyy + Vc * HUxyHVyy_y) +
                 ken5 * (Uc * UxxVxy + Vc * UxyVyy) + ken4 * (Uy * UxxVxy + Uc * UxxVxy_y + Vy * UxyVyy + Vc * UxyVyy_y) +
                 B2 * B2 * (DUx + DVy + reta * B2 * (Ux + Vy)) * (HUxyHVyy + ETAy * B2 * (Ux + Vy) + reta * B2 * UxyVyy);
    const T omega_0 = Vx - Uy;
    const T omega_1 = (b2 * rhx + B1 * ETAx) * B2 * (HUxyHVyy + (b2 * rh + B1 * reta) * B2 * UxyVyy) -
                      (b2 * rhy + B1 * ETAy) * B2 * (HUxxHVxy + (b2 * rh + B1 * reta) * B2 * UxxVxy);
    ken1 = ((B1 - one / two) * (reta + rh) * B2);
    ken2 = (one / (T)3 - B1 + half * B1 * B1) * rh * rh * B2 * B2 + (one / (T)6 - B1 + B1 * B1) * rh * reta * B2 +
           (one / two * B1 * B1 - one / (T)6) * reta * reta * B2 * B2;
    const T U3 = -Vc * omega_1 - omega_0 * (ken1 * HUxyHVyy + ken2 * UxyVyy);
    const T V3 = Uc * omega_1 + omega_0 * (ken1 * HUxxHVxy + ken2 * UxxVxy);
    f.Udisp[id] = U1pp + U2 + U3;
    f.Vdisp[id] = V1pp + V2 + V3;
}

// ---------------------------------------------------------------------------
// FLUXES (fluxes.F:52-117): 4th-order MUSCL-TVD (CONSTRUCT_HO_X/Y
// :1531-1754), Zhou wave speeds (:352-439), HLL (:171-194) and
// BOUNDARY_CONDITION (bc.F:53-295), fused per face.
// ---------------------------------------------------------------------------
template <typename T> __device__ __forceinline__ T lim3(T a, T b, T c) {
    if constexpr (sizeof(T) == sizeof(float)) {
        // s * max(0, min(|a|, 2 s b, 2 s c)), s = sign(a): the same value
        // without a branch, except that a zero result may carry the other
        // sign, which the float face values (harmonic means of products
        // tested > 0) never see
        const float s = a >= 0.0f ? 1.0f : -1.0f;
        return s * fmaxf(0.0f, fminf(fminf(fabsf(a), 2.0f * s * b), 2.0f * s * c));
    } else {
        // both arms, then a select: each thread gets the value of its arm
        // (signed zeros included) without the warp splitting on the sign
        const T pos = tmax((T)0, tmin(tmin(a, (T)2 * b), (T)2 * c));
        const T neg = tmin((T)0, tmax(tmax(a, (T)2 * b), (T)2 * c));
        return a >= (T)0 ? pos : neg;
    }
}
// Din(p) from v[0..3] = Vin(p-2..p+1), m[0..3] = MASK(p-2..p+1)
// (fluxes.F:1548-1598).  When any of the four cells is dry the reference
// either limits three equal slopes, which returns TXP2 for each of them, or
// zeroes the limited slopes; both give TXP2 - 1/6*(+0) = TXP2 exactly, so
// the limiter is only evaluated for four wet cells.
template <typename T> __device__ __forceinline__ T ho_din(const T *v, const int *m) {
    const T TXP1 = v[1] - v[0], TXP2 = v[2] - v[1], TXP3 = v[3] - v[2];
    if (!(m[0] && m[1] && m[2] && m[3])) return TXP2;
    const T DVP1 = lim3(TXP1, TXP2, TXP3), DVP2 = lim3(TXP2, TXP3, TXP1), DVP3 = lim3(TXP3, TXP1, TXP2);
    return TXP2 - (T)1 / (T)6 * (DVP3 - (T)2 * DVP2 + DVP1);
}
template <typename T> __device__ __forceinline__ T vl_guard(T t) {
    if (fabs_(t) <= (T)SMALL) t = (T)SMALL * fcopysign((T)1, t);
    return t;
}
template <typename T> __device__ __forceinline__ T vl_phi(T rat) {
    T van = (T)0;
    if (fabs_((T)1 + rat) > (T)SMALL) van = (rat + fabs_(rat)) / ((T)1 + rat);
    return van;
}
template <typename T> __device__ __forceinline__ T hll(T SL, T SR, T FL, T FR, T UL, T UR) {
    if (SL >= (T)0) return FL;
    if (SR <= (T)0) return FR;
    T f = SR * FL - SL * FR + SL * SR * (UR - UL);
    if (fabs_(SR - SL) < (T)SMALL) return f / (T)SMALL;
    return f / (SR - SL);
}
template <typename T> __device__ __forceinline__ T press(T Xi, T Deps, T g3) {
    return (T)0.5 * (T)GRAV * (Xi * Xi * g3 + (T)2 * Xi * Deps);
}

// Limited face values of one field from Din(p-1), Din(p), Din(p+1) and the
// cells p-1, p.  FP64 evaluates the reference's van Leer expressions
// (fluxes.F:1602-1630), including its guard that replaces a slope
// |t| <= SMALL by SMALL*sign(t).  The mixed path uses the equal closed form
// VAN1*TMP1 = VAN2*TMP2 = 2*TMP1*TMP2/(TMP1+TMP2) for TMP1*TMP2 > 0, else 0,
// without the guard (which only adds SMALL-sized corrections, e.g. on still
// water; the closed form needs no guard since TMP1*TMP2 > 0 keeps
// TMP1+TMP2 away from 0).
template <typename T>
__device__ __forceinline__ void ho_lr(T vm1, T v0, T d0, T d1, T d2, T &L, T &R) {
    if constexpr (sizeof(T) == sizeof(double)) {
        T t1 = vl_guard(d0), t2 = vl_guard(d1);
        T van1 = vl_phi(t2 / t1), van2 = vl_phi(t1 / t2);
        L = vm1 + ((T)1 / (T)6) * (van1 * t1 + (T)2 * van2 * t2);
        t1 = vl_guard(d1);
        t2 = vl_guard(d2);
        van1 = vl_phi(t2 / t1);
        van2 = vl_phi(t1 / t2);
        R = v0 - ((T)1 / (T)6) * ((T)2 * van1 * t1 + van2 * t2);
    } else {
        const T t1 = d0, t2 = d1, t3 = d2;
        const T hl = (t1 * t2 > (T)0) ? (T)2 * t1 * t2 / (t1 + t2) : (T)0;
        const T hr = (t2 * t3 > (T)0) ? (T)2 * t2 * t3 / (t2 + t3) : (T)0;
        L = vm1 + (T)0.5 * hl;
        R = v0 - (T)0.5 * hr;
    }
}

// Faces of direction DIR (0: x-faces, 1: y-faces).  A tile is 32 x FY
// faces, FY/8 per thread (by default 32 x 8 x-faces and 32 x 32 y-faces,
// so that the three-cell halo along y is shared by 32 faces; 32 x 16 in
// FP64; fw_autotune may pick another compiled height).  Din of the seven reconstructed fields is
// computed once per cell position into shared memory; each thread then
// finishes its faces: face values, Zhou wave speeds, HLL and the
// boundary/dry-face rules.  Normal velocity is U for x and V for y.
template <typename T, int DIR> constexpr int flux_fy_default() {
    return DIR == 0 ? 8 : (sizeof(T) == sizeof(double) ? 16 : 32);
}

template <typename T, int DIR, int FY_ = flux_fy_default<T, DIR>()> struct FluxTile {
    static constexpr int BX = 32, BY = 8;              // threads
    // faces of a tile (y tiles of doubles at most 16 high: 48 KB static shared memory)
    static constexpr int FX = 32, FY = FY_;
    static constexpr int FPT = FY / BY;                // faces per thread
    static constexpr int NB = DIR == 0 ? FX : FY;      // faces per tile line
    static constexpr int NTL = DIR == 0 ? FY : FX;     // tile lines
    static constexpr int NPOS = NB + 2;                // Din positions per line
    static constexpr int NP = DIR == 0 ? NPOS : NPOS + 1;  // odd row length for y
};

template <typename T, int DIR, int FY_ = flux_fy_default<T, DIR>()>
__global__ void __launch_bounds__(256) k_flux(Grid g, Fields<T> f) {
    using TL = FluxTile<T, DIR, FY_>;
    static_assert(TL::FY % TL::BY == 0, "whole faces per thread");
    constexpr int BX = TL::BX, BY = TL::BY, NTL = TL::NTL, NPOS = TL::NPOS, NP = TL::NP;
    __shared__ T din[7][NTL][NP];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int i0 = g.ib + blockIdx.x * TL::FX, j0 = g.jb + blockIdx.y * TL::FY;
    const int lo = DIR == 0 ? g.ib : g.jb, hi = DIR == 0 ? g.ie : g.je;
    const int base = (DIR == 0 ? i0 : j0) - 1;
    const T *src[7] = {f.U, f.V, f.HU, f.HV, f.Eta, f.U4, f.V4};
    const int nvar = g.dispersion ? 7 : 5;
    // 32-bit offsets: the arena planes hold fewer than 2^31 elements
    const int stride = DIR == 0 ? 1 : g.pitch;
    // the NTL x NPOS Din positions of the tile, spread over all threads
    // (consecutive threads on consecutive x for coalesced loads)
    const int tid = tx + ty * BX;
    for (int it = tid; it < NTL * NPOS; it += BX * BY) {
        const int k = DIR == 0 ? it % NPOS : it / NTL;
        const int ln = DIR == 0 ? it / NPOS : it % NTL;
        const int p = base + k;
        const int ci = DIR == 0 ? p : i0 + ln;
        const int cj = DIR == 0 ? j0 + ln : p;
        const bool lok = DIR == 0 ? (cj <= g.je) : (ci <= g.ie);
        if (lok && p >= lo - 1 && p <= hi + 2) {
            const int o0 = ci + cj * g.pitch - 2 * stride;
            int m[4];
#pragma unroll
            for (int q = 0; q < 4; q++) m[q] = ro(f.MASK + (o0 + q * stride));
#pragma unroll
            for (int vv = 0; vv < 7; vv++) {
                if (vv < nvar) {
                    T v[4];
#pragma unroll
                    for (int q = 0; q < 4; q++) v[q] = ro(src[vv] + (o0 + q * stride));
                    din[vv][ln][k] = ho_din(v, m);
                }
            }
        }
    }
    __syncthreads();
    const T g1 = GC(gamma1), g3 = GC(gamma3);
    for (int r = 0; r < TL::FPT; r++) {
    const int i = i0 + tx;
    const int j = j0 + ty + r * BY;
    if (DIR == 0) {
        if (i > g.ie + 1 || j > g.je) continue;
    } else {
        if (i > g.ie || j > g.je + 1) continue;
    }
    const int own = DIR == 0 ? tx : ty + r * BY;
    const int line = DIR == 0 ? ty + r * BY : tx;
    const int fid = i + j * g.pitch;
    const int cm = fid - stride;  // cell pos-1 (cell pos is fid)
    const int kf = own + 1;
    T Lv[7], Rv[7];
#pragma unroll
    for (int vv = 0; vv < 7; vv++) {
        if (vv >= nvar) {
            Lv[vv] = (T)0;
            Rv[vv] = (T)0;
            continue;
        }
        ho_lr(ro(src[vv] + (cm)), ro(src[vv] + (fid)), din[vv][line][kf - 1], din[vv][line][kf], din[vv][line][kf + 1], Lv[vv],
              Rv[vv]);
    }
    const T UL = Lv[0], UR = Rv[0], VL = Lv[1], VR = Rv[1], HUL = Lv[2], HUR = Rv[2];
    const T HVL = Lv[3], HVR = Rv[3], EL = Lv[4], ER = Rv[4];
    const T U4L = Lv[5], U4R = Rv[5], V4L = Lv[6], V4R = Rv[6];
    const T Dd = DIR == 0 ? ro(f.Depthx + (fid)) : ro(f.Depthy + (fid));
    const T HL = EL + Dd, HR = ER + Dd;
    // MASK9u(Mloc1,:) = MASK9(Mloc,:) (fluxes.F:1333); the faces computed
    // here never reach that column
    const T m9 = m2r<T>(ro(f.MASK9 + (fid)));
    const T nL = DIR == 0 ? UL : VL, nR = DIR == 0 ? UR : VR;
    const T tL = DIR == 0 ? VL : UL, tR = DIR == 0 ? VR : UR;
    const T n4L = DIR == 0 ? U4L : V4L, n4R = DIR == 0 ? U4R : V4R;
    const T t4L = DIR == 0 ? V4L : U4L, t4R = DIR == 0 ? V4R : U4R;
    const T qnL = DIR == 0 ? HUL : HVL, qnR = DIR == 0 ? HUR : HVR;  // HU for x, HV for y
    const T qtL = DIR == 0 ? HVL : HUL, qtR = DIR == 0 ? HVR : HUR;
    // mass flux PL/QL, normal momentum flux FxL/GyL, tangential GxL/FyL
    const T ML = qnL + g1 * m9 * HL * n4L;
    const T MR = qnR + g1 * m9 * HR * n4R;
    const T NL = g3 * ML * (nL + g1 * m9 * n4L) + (T)0.5 * (T)GRAV * ((EL) * (EL)*g3 + (T)2 * (EL) * (Dd));
    const T NR = g3 * MR * (nR + g1 * m9 * n4R) + (T)0.5 * (T)GRAV * ((ER) * (ER)*g3 + (T)2 * (ER) * (Dd));
    T TL, TR;
    if (DIR == 0) {
        TL = HL * (nL + g1 * m9 * n4L) * (tL + g1 * m9 * t4L) * g3;
        TR = HR * (nR + g1 * m9 * n4R) * (tR + g1 * m9 * t4R) * g3;
    } else {
        TL = HL * (tL + g1 * m9 * t4L) * (nL + g1 * m9 * n4L) * g3;
        TR = HR * (tR + g1 * m9 * t4R) * (nR + g1 * m9 * n4R) * g3;
    }
    // WAVE_SPEED (Zhou et al. 2001)
    const T SQR_PHI_L = fsqrt((T)GRAV * fabs_(HL));
    const T SQR_PHI_R = fsqrt((T)GRAV * fabs_(HR));
    const T SQR_PHI_S = (T)0.5 * (SQR_PHI_L + SQR_PHI_R) + (T)0.25 * (nL - nR);
    const T U_S = (T)0.5 * (nL + nR) + SQR_PHI_L - SQR_PHI_R;
    const T SL = tmin(nL - SQR_PHI_L, U_S - SQR_PHI_S);
    const T SR = tmax(nR + SQR_PHI_R, U_S + SQR_PHI_S);
    T Pm = hll(SL, SR, ML, MR, EL, ER);
    T Nm = hll(SL, SR, NL, NR, qnL, qnR);
    T Tm = hll(SL, SR, TL, TR, qtL, qtR);
    // BOUNDARY_CONDITION: walls, then the dry-cell loop (last write wins)
    const int pos = DIR == 0 ? i : j;
    const bool wall_on = DIR == 0 || !g.periodic;
    if (wall_on && pos == lo) {
        Pm = (T)0;
        Nm = press(ER, Dd, g3);
        Tm = (T)0;
    }
    if (wall_on && pos == hi + 1) {
        Pm = (T)0;
        Nm = press(EL, Dd, g3);
        Tm = (T)0;
    }
    const int mL = ro(f.MASK + (cm)), mR = ro(f.MASK + (fid));  // cells pos-1 and pos
    if (mL < 1) {
        Pm = (T)0;
        Nm = (pos - 1 != hi) ? press(ER, Dd, g3) * m2r<T>(mR) : (T)0;
        Tm = (T)0;
    }
    if (mR < 1) {
        Pm = (T)0;
        Nm = (pos != lo) ? press(EL, Dd, g3) * m2r<T>(mL) : (T)0;
        Tm = (T)0;
    }
    if (DIR == 0) {
        f.P[fid] = Pm;
        f.Fx[fid] = Nm;
        f.Gx[fid] = Tm;
    } else {
        f.Q[fid] = Pm;
        f.Gy[fid] = Nm;
        f.Fy[fid] = Tm;
    }
    }
}

// The tile's inputs staged by TMA: one 2-D tensor load of each of U V HU HV
// Eta U4 V4 (40 cells wide from i0 - 3, FY rows from j0 for x faces or FY+6
// rows from j0 - 3 for y faces) and of MASK (48 wide), completing on one
// mbarrier; Din and the faces then read shared memory.  i0 - 3 is a
// multiple of 32 (ib = 3), so every box starts on a 16-byte boundary.  The
// same arithmetic as k_flux, so the same results.
template <typename T, int DIR, int FY_> struct FluxStage {
    using TL = FluxTile<T, DIR, FY_>;
    static constexpr int BW = 40, BWM = 48;             // staged columns from i0 - 3
    static constexpr int BH = DIR == 0 ? FY_ : FY_ + 6;  // staged rows from j0 (x) or j0 - 3 (y)
    static constexpr int FB = (BW * BH * (int)sizeof(T) + 127) / 128 * 128;
    static constexpr int MB = (BWM * BH + 127) / 128 * 128;
    static constexpr int DB = (7 * TL::NTL * TL::NP * (int)sizeof(T) + 127) / 128 * 128;
    static constexpr int BYTES = 7 * FB + MB + DB + 16 + 128;
};

template <typename T> __device__ __forceinline__ T fnan();
template <> __device__ __forceinline__ float fnan<float>() { return __int_as_float(0x7fffffff); }
template <> __device__ __forceinline__ double fnan<double>() { return __longlong_as_double(0x7fffffffffffffffll); }

template <typename T, int DIR, int FY_>
__global__ void __launch_bounds__(256) k_flux_tma(Grid g, Fields<T> f, const __grid_constant__ FluxMaps maps) {
    using TL = FluxTile<T, DIR, FY_>;
    using S = FluxStage<T, DIR, FY_>;
    static_assert(TL::FY % TL::BY == 0, "whole faces per thread");
    constexpr int BX = TL::BX, BY = TL::BY, NTL = TL::NTL, NPOS = TL::NPOS, NP = TL::NP;
    extern __shared__ uint8_t fsm_raw[];
    uint8_t *sm = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(fsm_raw) + 127) & ~(uintptr_t)127);
    T(*din)[NTL][NP] = reinterpret_cast<T(*)[NTL][NP]>(sm + 7 * S::FB + S::MB);
    const uint32_t bar = fwtc::smem_u32(sm + 7 * S::FB + S::MB + S::DB);
#define FLD(v_, r_, c_) (reinterpret_cast<const T *>(sm + (v_) * S::FB)[(r_) * S::BW + (c_)])
#define MSK(r_, c_) ((int)(sm + 7 * S::FB)[(r_) * S::BWM + (c_)])
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int tid = tx + ty * BX;
    const int i0 = g.ib + blockIdx.x * TL::FX, j0 = g.jb + blockIdx.y * TL::FY;
    const int lo = DIR == 0 ? g.ib : g.jb, hi = DIR == 0 ? g.ie : g.je;
    const int base = (DIR == 0 ? i0 : j0) - 1;
    const int nvar = g.dispersion ? 7 : 5;
    if (tid == 0) {
        fwtc::mbar_init(bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (tid == 0) {
        const int xs = i0 - 3, ysr = DIR == 0 ? j0 : j0 - 3;
        fwtc::mbar_expect_tx(bar, (uint32_t)(nvar * S::BW * S::BH * (int)sizeof(T) + S::BWM * S::BH));
        for (int v = 0; v < nvar; v++) fwtc::tma_load_2d(fwtc::smem_u32(sm + v * S::FB), &maps.m[v], xs, ysr, bar);
        fwtc::tma_load_2d(fwtc::smem_u32(sm + 7 * S::FB), &maps.m[7], xs, ysr, bar);
    }
    const bool staged = fwtc::mbar_wait(bar, 0, maps.wait_limit ? maps.wait_limit : fwtc::WAIT_LIMIT);
    // the NTL x NPOS Din positions of the tile, spread over all threads
    for (int it = tid; it < NTL * NPOS; it += BX * BY) {
        const int k = DIR == 0 ? it % NPOS : it / NTL;
        const int ln = DIR == 0 ? it / NPOS : it % NTL;
        const int p = base + k;
        const int ci = DIR == 0 ? p : i0 + ln;
        const int cj = DIR == 0 ? j0 + ln : p;
        const bool lok = DIR == 0 ? (cj <= g.je) : (ci <= g.ie);
        if (lok && p >= lo - 1 && p <= hi + 2) {
            // cells p-2 .. p+1: staged columns k .. k+3 of row ln (x), or
            // rows k .. k+3 of column ln + 3 (y)
            int m[4];
#pragma unroll
            for (int q = 0; q < 4; q++) m[q] = DIR == 0 ? MSK(ln, k + q) : MSK(k + q, ln + 3);
#pragma unroll
            for (int vv = 0; vv < 7; vv++) {
                if (vv < nvar) {
                    T v[4];
#pragma unroll
                    for (int q = 0; q < 4; q++) v[q] = DIR == 0 ? FLD(vv, ln, k + q) : FLD(vv, k + q, ln + 3);
                    din[vv][ln][k] = ho_din(v, m);
                }
            }
        }
    }
    __syncthreads();
    const T g1 = GC(gamma1), g3 = GC(gamma3);
    for (int r = 0; r < TL::FPT; r++) {
    const int i = i0 + tx;
    const int j = j0 + ty + r * BY;
    if (DIR == 0) {
        if (i > g.ie + 1 || j > g.je) continue;
    } else {
        if (i > g.ie || j > g.je + 1) continue;
    }
    const int own = DIR == 0 ? tx : ty + r * BY;
    const int line = DIR == 0 ? ty + r * BY : tx;
    const int fid = i + j * g.pitch;
    const int kf = own + 1;
    T Lv[7], Rv[7];
#pragma unroll
    for (int vv = 0; vv < 7; vv++) {
        if (vv >= nvar) {
            Lv[vv] = (T)0;
            Rv[vv] = (T)0;
            continue;
        }
        // cells pos-1 and pos from the staged tile
        ho_lr(FLD(vv, DIR == 0 ? line : own + 2, DIR == 0 ? own + 2 : line + 3),
              FLD(vv, DIR == 0 ? line : own + 3, DIR == 0 ? own + 3 : line + 3), din[vv][line][kf - 1],
              din[vv][line][kf], din[vv][line][kf + 1], Lv[vv], Rv[vv]);
    }
    const T UL = Lv[0], UR = Rv[0], VL = Lv[1], VR = Rv[1], HUL = Lv[2], HUR = Rv[2];
    const T HVL = Lv[3], HVR = Rv[3], EL = Lv[4], ER = Rv[4];
    const T U4L = Lv[5], U4R = Rv[5], V4L = Lv[6], V4R = Rv[6];
    const T Dd = DIR == 0 ? ro(f.Depthx + (fid)) : ro(f.Depthy + (fid));
    const T HL = EL + Dd, HR = ER + Dd;
    // MASK9u(Mloc1,:) = MASK9(Mloc,:) (fluxes.F:1333); the faces computed
    // here never reach that column
    const T m9 = m2r<T>(ro(f.MASK9 + (fid)));
    const T nL = DIR == 0 ? UL : VL, nR = DIR == 0 ? UR : VR;
    const T tL = DIR == 0 ? VL : UL, tR = DIR == 0 ? VR : UR;
    const T n4L = DIR == 0 ? U4L : V4L, n4R = DIR == 0 ? U4R : V4R;
    const T t4L = DIR == 0 ? V4L : U4L, t4R = DIR == 0 ? V4R : U4R;
    const T qnL = DIR == 0 ? HUL : HVL, qnR = DIR == 0 ? HUR : HVR;  // HU for x, HV for y
    const T qtL = DIR == 0 ? HVL : HUL, qtR = DIR == 0 ? HVR : HUR;
    // mass flux PL/QL, normal momentum flux FxL/GyL, tangential GxL/FyL
    const T ML = qnL + g1 * m9 * HL * n4L;
    const T MR = qnR + g1 * m9 * HR * n4R;
    const T NL = g3 * ML * (nL + g1 * m9 * n4L) + (T)0.5 * (T)GRAV * ((EL) * (EL)*g3 + (T)2 * (EL) * (Dd));
    const T NR = g3 * MR * (nR + g1 * m9 * n4R) + (T)0.5 * (T)GRAV * ((ER) * (ER)*g3 + (T)2 * (ER) * (Dd));
    T TL, TR;
    if (DIR == 0) {
        TL = HL * (nL + g1 * m9 * n4L) * (tL + g1 * m9 * t4L) * g3;
        TR = HR * (nR + g1 * m9 * n4R) * (tR + g1 * m9 * t4R) * g3;
    } else {
        TL = HL * (tL + g1 * m9 * t4L) * (nL + g1 * m9 * n4L) * g3;
        TR = HR * (tR + g1 * m9 * t4R) * (nR + g1 * m9 * n4R) * g3;
    }
    // WAVE_SPEED (Zhou et al. 2001)
    const T SQR_PHI_L = fsqrt((T)GRAV * fabs_(HL));
    const T SQR_PHI_R = fsqrt((T)GRAV * fabs_(HR));
    const T SQR_PHI_S = (T)0.5 * (SQR_PHI_L + SQR_PHI_R) + (T)0.25 * (nL - nR);
    const T U_S = (T)0.5 * (nL + nR) + SQR_PHI_L - SQR_PHI_R;
    const T SL = tmin(nL - SQR_PHI_L, U_S - SQR_PHI_S);
    const T SR = tmax(nR + SQR_PHI_R, U_S + SQR_PHI_S);
    T Pm = hll(SL, SR, ML, MR, EL, ER);
    T Nm = hll(SL, SR, NL, NR, qnL, qnR);
    T Tm = hll(SL, SR, TL, TR, qtL, qtR);
    // BOUNDARY_CONDITION: walls, then the dry-cell loop (last write wins)
    const int pos = DIR == 0 ? i : j;
    const bool wall_on = DIR == 0 || !g.periodic;
    if (wall_on && pos == lo) {
        Pm = (T)0;
        Nm = press(ER, Dd, g3);
        Tm = (T)0;
    }
    if (wall_on && pos == hi + 1) {
        Pm = (T)0;
        Nm = press(EL, Dd, g3);
        Tm = (T)0;
    }
    const int mL = MSK(DIR == 0 ? line : own + 2, DIR == 0 ? own + 2 : line + 3);  // cell pos-1
    const int mR = MSK(DIR == 0 ? line : own + 3, DIR == 0 ? own + 3 : line + 3);  // cell pos
    if (mL < 1) {
        Pm = (T)0;
        Nm = (pos - 1 != hi) ? press(ER, Dd, g3) * m2r<T>(mR) : (T)0;
        Tm = (T)0;
    }
    if (mR < 1) {
        Pm = (T)0;
        Nm = (pos != lo) ? press(EL, Dd, g3) * m2r<T>(mL) : (T)0;
        Tm = (T)0;
    }
    if (!staged) {  // the tile never arrived: poison the fluxes (the step reports NaN)
        Pm = Nm = Tm = fnan<T>();
    }
    if (DIR == 0) {
        f.P[fid] = Pm;
        f.Fx[fid] = Nm;
        f.Gx[fid] = Tm;
    } else {
        f.Q[fid] = Pm;
        f.Gy[fid] = Nm;
        f.Fy[fid] = Tm;
    }
    }
    // the tile never arrived: its copies may still be in flight; one more
    // bounded wait (the full limit) keeps this block's shared memory until
    // they land
    if (!staged && tid == 0) fwtc::mbar_wait(bar, 0, fwtc::WAIT_LIMIT);
}

#undef FLD
#undef MSK

// ---------------------------------------------------------------------------
// SourceTerms (sources.F:56-548) at one interior cell, with the wavemaker
// mass of WK_REG / JON_2D (sources.F:109-134).
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ T wavemaker_mass(const Grid &g, const Fields<T> &f, int i, int j, double TIME) {
    if (i < g.ilo || i > g.ihi || j < g.jlo || j > g.jhi) return (T)0;
    if constexpr (sizeof(T) == sizeof(double)) {
        if (g.wavemaker == FW_WK_REG) {
            const T AA = ftanh((T)PI_SP / ((T)g.time_ramp * (T)g.tperiod) * (T)TIME) * (T)g.D_gen;
            const T xmk = (T)(i - g.ib) * (T)g.DX, ymk = (T)(j - g.jb) * (T)g.DY;
            const T dxm = xmk - (T)g.xc_wk;
            return AA * fexp(-(T)g.beta_gen * (dxm * dxm)) *
                   fsin((T)g.rlamda * (ymk - (T)0) - (T)2 * (T)PI_SP / (T)g.tperiod * (T)TIME);
        }
        if (g.wavemaker == FW_WK_JON_2D) {
            const T AA = ftanh((T)PI_SP / ((T)g.time_ramp / (T)g.freq_peak) * (T)TIME);
            const int bw = g.ihi - g.ilo + 1, bh = g.jhi - g.jlo + 1;
            const size_t b = (size_t)(i - g.ilo) + (size_t)(j - g.jlo) * bw;
            T s = (T)0;
            for (int k = 0; k < g.nfreq; k++)
                s = s + AA * ((T)f.Cm[b + (size_t)k * bw * bh] * (T)f.wmcs[2 * k] +
                              (T)f.Sm[b + (size_t)k * bw * bh] * (T)f.wmcs[2 * k + 1]);
            return s;
        }
    } else {
        // mixed: the ramp and phase of this step come from k_dt_final
        const T AA = f.fsc[FS_WKAA];
        if (g.wavemaker == FW_WK_REG) {
            const T xmk = i2r<T>(i - g.ib) * g.f_DX, ymk = i2r<T>(j - g.jb) * g.f_DY;
            const T dxm = xmk - g.f_xc_wk;
            return AA * fexp(-g.f_beta_gen * (dxm * dxm)) * fsin(g.f_rlamda * ymk - f.fsc[FS_WKPH]);
        }
        if (g.wavemaker == FW_WK_JON_2D) {
            const int bw = g.ihi - g.ilo + 1, bh = g.jhi - g.jlo + 1;
            const size_t b = (size_t)(i - g.ilo) + (size_t)(j - g.jlo) * bw;
            T s = (T)0;
            for (int k = 0; k < g.nfreq; k++)
                s = s + AA * ((T)f.Cm[b + (size_t)k * bw * bh] * f.wmcsf[2 * k] +
                              (T)f.Sm[b + (size_t)k * bw * bh] * f.wmcsf[2 * k + 1]);
            return s;
        }
    }
    return (T)0;
}

// SourceTerms at one cell; BX, BY get BreakSourceX/Y (sources.F:428-456),
// zero without viscosity breaking
template <typename T>
__device__ __forceinline__ void source_terms_b(const Grid &g, const Fields<T> &f, int i, int j, T wm, T &SX,
                                               T &SY, T &BX, T &BY) {
    BX = (T)0;
    BY = (T)0;
    constexpr bool EXACT = sizeof(T) == sizeof(double);
    const T DX = GC(DX), DY = GC(DY), mdf = GC(min_depth_frc);
    const T rdx = GC(rdx), rdy = GC(rdy);
    // x/DX: the reference's division in FP64, a reciprocal in the mixed path
#define OX(x) (EXACT ? (x) / DX : (x) * rdx)
#define OY(x) (EXACT ? (x) / DY : (x) * rdy)
    const T g1 = GC(gamma1), g2 = GC(gamma2);
    const size_t id = IDX(i, j);
    const size_t ie_ = IDX(i + 1, j), iw = IDX(i - 1, j), in_ = IDX(i, j + 1), is = IDX(i, j - 1);
    const T U = ro(f.U + (id)), V = ro(f.V + (id));
    const T spd = fsqrt(U * U + V * V);
    const T m9 = m2r<T>(ro(f.MASK9 + (id)));
    const T mk = m2r<T>(ro(f.MASK + (id)));
    const T Hm = tmax(f.H[id], mdf);
    const T Eta = f.Eta[id];
    const T U4 = ro(f.U4 + (id)), V4 = ro(f.V4 + (id));
    const T dPQ = OX(ro(f.P + (ie_)) - ro(f.P + (id))) + OY(ro(f.Q + (in_)) - ro(f.Q + (id)));
    const T FrcInsX = -ro(f.Cd + (id)) * U * spd;
    T sx = OX((T)GRAV * (Eta)) * (ro(f.Depthx + (ie_)) - ro(f.Depthx + (id))) * mk + FrcInsX +
           g1 * m9 * Hm *
               (OX(U * (T)0.5 * (ro(f.U4 + (ie_)) - ro(f.U4 + (iw)))) + OY(V * (T)0.5 * (ro(f.U4 + (in_)) - ro(f.U4 + (is)))) +
                OX(U4 * (T)0.5 * (ro(f.U + (ie_)) - ro(f.U + (iw)))) + OY(V4 * (T)0.5 * (ro(f.U + (in_)) - ro(f.U + (is)))) -
                g2 * m9 * ro(f.Udisp + (id))) +
           g1 * m9 * dPQ * (U4 - ro(f.U1p + (id))) + wm * U;
    const T FrcInsY = -ro(f.Cd + (id)) * V * spd;
    T sy = OY((T)GRAV * (Eta)) * (ro(f.Depthy + (in_)) - ro(f.Depthy + (id))) * mk + FrcInsY +
           g1 * m9 * Hm *
               (OX(U * (T)0.5 * (ro(f.V4 + (ie_)) - ro(f.V4 + (iw)))) + OY(V * (T)0.5 * (ro(f.V4 + (in_)) - ro(f.V4 + (is)))) +
                OX(U4 * (T)0.5 * (ro(f.V + (ie_)) - ro(f.V + (iw)))) + OY(V4 * (T)0.5 * (ro(f.V + (in_)) - ro(f.V + (is)))) -
                g2 * m9 * ro(f.Vdisp + (id))) +
           g1 * m9 * dPQ * (V4 - ro(f.V1p + (id))) + wm * V;
    if (g.friction_sponge) {
        sx = sx - ro(f.CD4 + (id)) * U * spd * ro(f.Depth + (id));
        sy = sy - ro(f.CD4 + (id)) * V * spd * ro(f.Depth + (id));
    }
    if (g.visc_breaking) {
        // nu_vis is a float array (sources.F:69): the face sums are float sums
        const float nc = (float)ro(f.nu + (id));
        const T nxp = (T)((float)ro(f.nu + (ie_)) + nc), nxm = (T)((float)ro(f.nu + (iw)) + nc);
        const T nyp = (T)((float)ro(f.nu + (in_)) + nc), nym = (T)((float)ro(f.nu + (is)) + nc);
        const T HUc = ro(f.HU + (id)), HVc = ro(f.HV + (id));
        T bx, by;
        if constexpr (EXACT) {
            bx = (T)0.5 / DX * (nxp * (T)1 / DX * (ro(f.HU + (ie_)) - HUc) - nxm * (T)1 / DX * (HUc - ro(f.HU + (iw)))) +
                 (T)0.5 / DY * (nyp * (T)1 / DY * (ro(f.HU + (in_)) - HUc) - nym * (T)1 / DY * (HUc - ro(f.HU + (is))));
            by = (T)0.5 / DX * (nxp * (T)1 / DX * (ro(f.HV + (ie_)) - HVc) - nxm * (T)1 / DX * (HVc - ro(f.HV + (iw)))) +
                 (T)0.5 / DY * (nyp * (T)1 / DY * (ro(f.HV + (in_)) - HVc) - nym * (T)1 / DY * (HVc - ro(f.HV + (is))));
        } else {
            const T cx = (T)g.f_cx, cy = (T)g.f_cy;
            bx = cx * (nxp * (ro(f.HU + (ie_)) - HUc) - nxm * (HUc - ro(f.HU + (iw)))) +
                 cy * (nyp * (ro(f.HU + (in_)) - HUc) - nym * (HUc - ro(f.HU + (is))));
            by = cx * (nxp * (ro(f.HV + (ie_)) - HVc) - nxm * (HVc - ro(f.HV + (iw)))) +
                 cy * (nyp * (ro(f.HV + (in_)) - HVc) - nym * (HVc - ro(f.HV + (is))));
        }
        sx = sx + bx;
        sy = sy + by;
        BX = bx;
        BY = by;
    }
#undef OX
#undef OY
    SX = sx;
    SY = sy;
}
template <typename T>
__device__ __forceinline__ void source_terms(const Grid &g, const Fields<T> &f, int i, int j, T wm, T &SX,
                                             T &SY) {
    T bx, by;
    source_terms_b(g, f, i, j, wm, SX, SY, bx, by);
}

// SourceTerms alone (materialises SourceX, SourceY, WaveMaker_Mass)
template <typename T>
__global__ void __launch_bounds__(256) k_sources(Grid g, Fields<T> f) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x + g.ib;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + g.jb;
    if (i > g.ie || j > g.je) return;
    const T wm = wavemaker_mass(g, f, i, j, f.dsc[S_TIME]);
    T sx, sy;
    source_terms(g, f, i, j, wm, sx, sy);
    f.SourceX[IDX(i, j)] = sx;
    f.SourceY[IDX(i, j)] = sy;
    f.WM[IDX(i, j)] = wm;
}

// ---------------------------------------------------------------------------
// ESTIMATE_HUV (etauv_solver.F:53-351) fused with SourceTerms, plus the H
// update and the right-hand sides of the tridiagonal systems of
// GET_Eta_U_V_HU_HV (etauv_solver.F:365-539).  RAD (the last two stages,
// with the radiation sums on) also stores P_center, Q_center, U_davg, V_davg
// with the stage's starting H (etauv_solver.F:94-101), Wsurf = R1
// (etauv_solver.F:247) and BreakSourceX/Y.
// ---------------------------------------------------------------------------
template <typename T, bool RAD = false>
__global__ void __launch_bounds__(256, sizeof(T) == sizeof(float) ? 4 : 3) k_update(Grid g, Fields<T> f, T al, T be) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= g.Mloc || j >= g.Nloc) return;
    const size_t id = IDX(i, j);
    const T g3 = GC(gamma3);
    if (i < g.ib || i > g.ie || j < g.jb || j > g.je) {
        f.H[id] = f.Eta[id] * g3 + ro(f.Depth + (id));  // H = Eta*Gamma3+Depth on all cells
        return;
    }
    if constexpr (sizeof(T) == sizeof(float)) {
        // the right-hand sides' inputs (rows j-1..j+1 of U, V, Depth, the
        // masks), read after this kernel's stores
        if (g.dispersion) {
#pragma unroll
            for (int b = -1; b <= 1; b++) {
                prefetch_l1(f.U + IDX(i, j + b));
                prefetch_l1(f.V + IDX(i, j + b));
                prefetch_l1(f.Depth + IDX(i, j + b));
            }
            prefetch_l1(f.MASK9 + id);
            prefetch_l1(f.MASK + id);
        }
    }
    const T DX = GC(DX), DY = GC(DY);
    const T DT = DTV;
    const double TIME = f.dsc[S_TIME];
    const T wm = wavemaker_mass(g, f, i, j, TIME);
    T SX, SY, BX, BY;
    source_terms_b(g, f, i, j, wm, SX, SY, BX, BY);

    const size_t ie_ = IDX(i + 1, j), in_ = IDX(i, j + 1);
    constexpr bool EXACT = sizeof(T) == sizeof(double);
    const T cdx = EXACT ? (T)1 / DX : GC(rdx), cdy = EXACT ? (T)1 / DY : GC(rdy);
    T R1 = -cdx * (ro(f.P + (ie_)) * (T)1 + ro(f.P + (id)) * (T)-1) - cdy * (ro(f.Q + (in_)) * (T)1 + ro(f.Q + (id)) * (T)-1);
    if (g.wavemaker != FW_WK_NONE) {
        const T xmk = i2r<T>(i - g.ib) * DX, ymk = i2r<T>(j - g.jb) * DY;
        if (fabs_(xmk - GC(xc_wk)) < GC(width_wk) && fabs_(ymk - GC(yc_wk)) < GC(ywidth_wk) / (T)2)
            R1 = R1 + wm;
    }
    if constexpr (RAD) {
        const size_t PL = (size_t)g.pitch * (size_t)(g.Nloc + 1);
        const T pc = (T)0.5 * (ro(f.P + (ie_)) + ro(f.P + (id))), qc = (T)0.5 * (ro(f.Q + (in_)) + ro(f.Q + (id)));
        const T hm = tmax(f.H[id], GC(min_depth_frc));  // H before this stage's update
        f.rad[RP_PC * PL + id] = pc;
        f.rad[RP_QC * PL + id] = qc;
        f.rad[RP_UD * PL + id] = pc / hm;
        f.rad[RP_VD * PL + id] = qc / hm;
        f.rad[RP_WS * PL + id] = R1;
        f.rad[RP_BX * PL + id] = BX;
        f.rad[RP_BY * PL + id] = BY;
    }
    T eta = al * ro(f.Eta0 + (id)) + be * (f.Eta[id] + DT * R1);
    if (g.eta_limiter) {
        if (eta < GC(trough)) eta = GC(trough);
        if (eta > GC(crest)) eta = GC(crest);
    }
    const T R2 = -cdx * (ro(f.Fx + (ie_)) * (T)1 + ro(f.Fx + (id)) * (T)-1) - cdy * (ro(f.Fy + (in_)) * (T)1 + ro(f.Fy + (id)) * (T)-1) + SX;
    const T ubar = al * ro(f.Ubar0 + (id)) + be * (f.Ubar[id] + DT * R2);
    const T R3 = -cdx * (ro(f.Gx + (ie_)) * (T)1 + ro(f.Gx + (id)) * (T)-1) - cdy * (ro(f.Gy + (in_)) * (T)1 + ro(f.Gy + (id)) * (T)-1) + SY;
    const T vbar = al * ro(f.Vbar0 + (id)) + be * (f.Vbar[id] + DT * R3);
    f.Eta[id] = eta;
    f.Ubar[id] = ubar;
    f.Vbar[id] = vbar;
    const T H = eta * g3 + ro(f.Depth + (id));
    f.H[id] = H;
    if (!g.dispersion) return;

    // tmp4 of the x and y systems (etauv_solver.F:410-411, 508-509)
    if constexpr (sizeof(T) == sizeof(double)) {
        const double mdf = g.min_depth_frc;
        const double g1 = g.gamma1, b1 = g.b1, b2 = g.b2;
        const double m9 = (double)ro(f.MASK9 + (id));
        const double mk = (double)ro(f.MASK + (id));
        const double dep = tmax((double)ro(f.Depth + (id)), mdf);
        const double Hm = tmax((double)H, mdf);
        // the cross derivatives CAL_DISPERSION left at the start of the stage
        const double Vxy = ro(f.Vxy + (id)), DVxy = ro(f.DVxy + (id)), Uxy = ro(f.Uxy + (id)), DUxy = ro(f.DUxy + (id));
        f.rhs_x[id] = (double)ubar * mk / Hm + g1 * m9 * (-b1 / 2.0 * dep * dep * Vxy - b2 * dep * DVxy);
        f.rhs_y[id] = (double)vbar * mk / Hm + g1 * m9 * (-b1 / 2.0 * dep * dep * Uxy - b2 * dep * DUxy);
    } else {
        // mixed: float arithmetic; the cross derivatives of the stage-start
        // U, V are recomputed here
        const T mf = g.f_min_depth_frc;
        const T m9 = m2r<T>(ro(f.MASK9 + (id))), mk = m2r<T>(ro(f.MASK + (id)));
        const T dep = tmax(ro(f.Depth + (id)), mf);
        const bool wall = (i == g.ib) || (i == g.ie) || (j == g.jb) || (j == g.je);
        T Vxy = (T)0, DVxy = (T)0, Uxy = (T)0, DUxy = (T)0;
        if (!wall) {
            const T q = g.f_rdxy4 * m9;
#define XY(F) (((F(1, 1) - F(1, -1)) - (F(-1, 1) - F(-1, -1))) * q)
#define LV(a, b) (ro(f.V + (IDX(i + (a), j + (b)))))
#define LU(a, b) (ro(f.U + (IDX(i + (a), j + (b)))))
#define LDV(a, b) (tmax(ro(f.Depth + (IDX(i + (a), j + (b)))), mf) * LV(a, b))
#define LDU(a, b) (tmax(ro(f.Depth + (IDX(i + (a), j + (b)))), mf) * LU(a, b))
            Vxy = XY(LV);
            DVxy = XY(LDV);
            Uxy = XY(LU);
            DUxy = XY(LDU);
#undef XY
#undef LV
#undef LU
#undef LDV
#undef LDU
        }
        const T fg = g.f_gamma1 * m9, rH = (T)1 / tmax(H, mf);
        f.rhs_x[id] = ubar * mk * rH + fg * (g.f_hb1 * dep * dep * Vxy - g.f_b2 * dep * DVxy);
        f.rhs_y[id] = vbar * mk * rH + fg * (g.f_hb1 * dep * dep * Uxy - g.f_b2 * dep * DUxy);
    }
}

// ---------------------------------------------------------------------------
// Tridiagonal u/v recovery (TRIDx_ser / TRIDy_ser / TRIDy_periodic,
// tridiagnal.F:59-398) as a partitioned line solver in double:
//   A: every chunk of m rows eliminates its interior rows for three right-
//      hand sides and emits two rows of a reduced tridiagonal system;
//   B: one thread per line solves the reduced system (two right-hand sides
//      and the Sherman-Morrison combination for periodic y);
//   C: every chunk back-substitutes its interior rows.
// Rows are the reference's normalised rows a x(k-1) + x(k) + c x(k+1) = d.
// ---------------------------------------------------------------------------
template <typename T, int DIR>
__device__ __forceinline__ void tri_coef(const Grid &g, const Fields<T> &f, int i, int j, double &a, double &c,
                                         double &d) {
    const double mdf = g.min_depth_frc, g1 = g.gamma1;
    const size_t id = IDX(i, j);
    const double dep = tmax((double)f.Depth[id], mdf);
    const double depl = tmax((double)f.Depth[DIR == 0 ? IDX(i - 1, j) : IDX(i, j - 1)], mdf);
    const double depr = tmax((double)f.Depth[DIR == 0 ? IDX(i + 1, j) : IDX(i, j + 1)], mdf);
    const double m9 = (double)f.MASK9[id];
    const double tmp4 = DIR == 0 ? f.rhs_x[id] : f.rhs_y[id];
    double tmp1, tmp2, tmp3;
    if constexpr (sizeof(T) == sizeof(double)) {
        // the reference's expressions (etauv_solver.F:406-409, 504-507);
        // their constant left parts (b1 / 2.0 / h / h and so on) come
        // evaluated in the same order
        const double k1 = g.tK1[DIR], k2 = g.tK2[DIR], k3 = g.tK3[DIR], k4 = g.tK4[DIR];
        tmp1 = g1 * m9 * (k1 * dep * dep + k2 * depl * dep);
        tmp2 = 1.0 + g1 * m9 * (k3 * dep * dep - k4 * dep * dep);
        tmp3 = g1 * m9 * (k1 * dep * dep + k2 * dep * depr);
        if (tmp2 != 0.0 || f.MASK[id] > 0) {
            a = tmp1 / tmp2;
            c = tmp3 / tmp2;
            d = tmp4 / tmp2;
        } else {
            a = 0.0;
            c = 0.0;
            d = 0.0;
        }
    } else {
        // mixed: the same coefficients from per-direction constants and one
        // reciprocal
        const double gm = g1 * m9;
        tmp1 = gm * dep * (g.cA[DIR] * dep + g.cB[DIR] * depl);
        tmp2 = 1.0 + gm * g.cC[DIR] * dep * dep;
        tmp3 = gm * dep * (g.cA[DIR] * dep + g.cB[DIR] * depr);
        if (tmp2 != 0.0 || f.MASK[id] > 0) {
            const double r = 1.0 / tmp2;
            a = tmp1 * r;
            c = tmp3 * r;
            d = tmp4 * r;
        } else {
            a = 0.0;
            c = 0.0;
            d = 0.0;
        }
    }
}

// row k (0..L-1) of line l -> cell
template <int DIR> __device__ __forceinline__ void line_cell(const Grid &g, int l, int k, int &i, int &j) {
    if (DIR == 0) {
        i = g.ib + k;
        j = g.jb + l;
    } else {
        i = g.ib + l;
        j = g.jb + k;
    }
}

// coefficients of row k of line l, with the periodic end-row scaling of
// TRIDy_periodic (tridiagnal.F:168-173) when PER
template <typename T, int DIR, bool PER>
__device__ __forceinline__ void row_coef(const Grid &g, const Fields<T> &f, const LinePart &lp, int l, int k,
                                         double &a, double &c, double &d) {
    int i, j;
    line_cell<DIR>(g, l, k, i, j);
    tri_coef<T, DIR>(g, f, i, j, a, c, d);
    if (PER) {
        if (k == 0) {
            double a2, c2, d2;
            int ie2, je2;
            line_cell<DIR>(g, l, lp.L - 1, ie2, je2);
            tri_coef<T, DIR>(g, f, ie2, je2, a2, c2, d2);  // c_end
            c = c / (1 + c2);
            d = d / (1 + c2);
        } else if (k == lp.L - 1) {
            double a2, c2, d2;
            int ib2, jb2;
            line_cell<DIR>(g, l, 0, ib2, jb2);
            tri_coef<T, DIR>(g, f, ib2, jb2, a2, c2, d2);  // a_beg
            a = a / (1 + a2);
            d = d / (1 + a2);
        }
    }
}

template <int DIR>
__device__ __forceinline__ void chunk_of(const LinePart &lp, int t, int &l, int &ch) {
    // x lines: consecutive threads walk the chunks of one line;
    // y lines: consecutive threads walk neighbouring lines (coalesced)
    if (DIR == 0) {
        l = t / lp.P;
        ch = t % lp.P;
    } else {
        ch = t / lp.nlines;
        l = t % lp.nlines;
    }
}

template <typename T, int DIR, bool PER>
__global__ void __launch_bounds__(128) k_tri_a(Grid g, Fields<T> f, LinePart lp) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= lp.nlines * lp.P) return;
    int l, ch;
    chunk_of<DIR>(lp, t, l, ch);
    const int s = ch * lp.m;
    const int e = (ch == lp.P - 1) ? lp.L - 1 : s + lp.m - 1;
    double as, cs, ds, ae, ce, de;
    row_coef<T, DIR, PER>(g, f, lp, l, s, as, cs, ds);
    row_coef<T, DIR, PER>(g, f, lp, l, e, ae, ce, de);
    if (s == 0) as = 0.0;           // first row: no lower neighbour
    if (e == lp.L - 1) ce = 0.0;    // last row: no upper neighbour
    double lo_s, di_s, up_s, r_s, lo_e, di_e, up_e, r_e;
    if (e - s >= 2) {
        // interior rows s+1..e-1: forward sweep with three right-hand sides
        double cp = 0.0, yp = 0.0, pp = 0.0, qp = 0.0;
        for (int k = s + 1; k <= e - 1; k++) {
            double a, c, d;
            row_coef<T, DIR, PER>(g, f, lp, l, k, a, c, d);
            const double lower = (k > s + 1) ? a : 0.0;
            const double r = 1.0 / (1.0 - lower * cp);
            const double upper = (k < e - 1) ? c : 0.0;
            cp = upper * r;
            yp = (d - lower * yp) * r;
            pp = ((k == s + 1 ? a : 0.0) - lower * pp) * r;
            qp = ((k == e - 1 ? c : 0.0) - lower * qp) * r;
            int ii, jj;
            line_cell<DIR>(g, l, k, ii, jj);
            const size_t q = IDX(ii, jj);
            f.ty[q] = yp;
            f.tp[q] = pp;
            f.tq[q] = qp;
            f.tc[q] = cp;  // c' for the backward sweep
        }
        // backward sweep
        double yn = 0.0, pn = 0.0, qn = 0.0;
        double y1 = 0, p1 = 0, q1 = 0, yl = 0, pl = 0, ql = 0;
        for (int k = e - 1; k >= s + 1; k--) {
            int ii, jj;
            line_cell<DIR>(g, l, k, ii, jj);
            const size_t q = IDX(ii, jj);
            const double cpk = f.tc[q];
            const double yk = f.ty[q] - cpk * yn;
            const double pk = f.tp[q] - cpk * pn;
            const double qk = f.tq[q] - cpk * qn;
            f.ty[q] = yk;
            f.tp[q] = pk;
            f.tq[q] = qk;
            yn = yk;
            pn = pk;
            qn = qk;
            if (k == e - 1) {
                yl = yk;
                pl = pk;
                ql = qk;
            }
            if (k == s + 1) {
                y1 = yk;
                p1 = pk;
                q1 = qk;
            }
        }
        lo_s = as;
        di_s = 1.0 - cs * p1;
        up_s = -cs * q1;
        r_s = ds - cs * y1;
        lo_e = -ae * pl;
        di_e = 1.0 - ae * ql;
        up_e = ce;
        r_e = de - ae * yl;
    } else {
        lo_s = as;
        di_s = 1.0;
        up_s = cs;
        r_s = ds;
        lo_e = ae;
        di_e = 1.0;
        up_e = ce;
        r_e = de;
    }
    double *red = f.red + ((size_t)l * 2 * lp.P + 2 * ch) * 6;
    red[0] = lo_s;
    red[1] = di_s;
    red[2] = up_s;
    red[3] = r_s;
    red[4] = (PER && s == 0) ? 1.0 : 0.0;  // second right-hand side (scaled below)
    red[6 + 0] = lo_e;
    red[6 + 1] = di_e;
    red[6 + 2] = up_e;
    red[6 + 3] = r_e;
    red[6 + 4] = (PER && e == lp.L - 1) ? 1.0 : 0.0;
}

template <typename T, int DIR, bool PER>
__global__ void __launch_bounds__(128) k_tri_b(Grid g, Fields<T> f, LinePart lp) {
    const int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= lp.nlines) return;
    const int n = 2 * lp.P;
    double *red = f.red + (size_t)l * n * 6;
    double a_beg = 0.0, c_end = 0.0;
    if (PER) {
        double a, c, d;
        int i, j;
        line_cell<DIR>(g, l, 0, i, j);
        tri_coef<T, DIR>(g, f, i, j, a, c, d);
        a_beg = a;
        line_cell<DIR>(g, l, lp.L - 1, i, j);
        tri_coef<T, DIR>(g, f, i, j, a, c, d);
        c_end = c;
        // e = [1/(1+c_end), 0, ..., 0, -1/(1+a_beg)] (tridiagnal.F:207-215)
        red[4] = 1.0 / (1.0 + c_end);
        red[(size_t)(n - 1) * 6 + 4] = -1.0 / (1.0 + a_beg);
    }
    // Thomas on the reduced rows: slot 5 keeps c', slots 3/4 the rhs
    double cp = 0.0, r1 = 0.0, r2 = 0.0;
    for (int k = 0; k < n; k++) {
        double *row = red + (size_t)k * 6;
        const double lo = (k > 0) ? row[0] : 0.0;
        const double den = row[1] - lo * cp;
        cp = (k < n - 1 ? row[2] : 0.0) / den;
        r1 = (row[3] - lo * r1) / den;
        row[5] = cp;
        row[3] = r1;
        if (PER) {
            r2 = (row[4] - lo * r2) / den;
            row[4] = r2;
        }
    }
    double x1 = 0.0, x2 = 0.0;
    for (int k = n - 1; k >= 0; k--) {
        double *row = red + (size_t)k * 6;
        x1 = row[3] - row[5] * x1;
        row[3] = x1;
        if (PER) {
            x2 = row[4] - row[5] * x2;
            row[4] = x2;
        }
    }
    if (PER) {
        const double y1b = red[3], y1e = red[(size_t)(n - 1) * 6 + 3];
        const double y2b = red[4], y2e = red[(size_t)(n - 1) * 6 + 4];
        const double beta = (c_end * y1b - a_beg * y1e) / (1.0 - (c_end * y2b - a_beg * y2e));
        for (int k = 0; k < n; k++) {
            double *row = red + (size_t)k * 6;
            row[3] = row[3] + beta * row[4];
        }
    }
}

template <typename T, int DIR>
__global__ void __launch_bounds__(128) k_tri_c(Grid g, Fields<T> f, LinePart lp) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= lp.nlines * lp.P) return;
    int l, ch;
    chunk_of<DIR>(lp, t, l, ch);
    const int s = ch * lp.m;
    const int e = (ch == lp.P - 1) ? lp.L - 1 : s + lp.m - 1;
    const double *red = f.red + ((size_t)l * 2 * lp.P + 2 * ch) * 6;
    const double xs = red[3], xe = red[6 + 3];
    T *out = DIR == 0 ? f.U : f.V;
    int i, j;
    line_cell<DIR>(g, l, s, i, j);
    out[IDX(i, j)] = (T)xs;
    line_cell<DIR>(g, l, e, i, j);
    out[IDX(i, j)] = (T)xe;
    for (int k = s + 1; k <= e - 1; k++) {
        line_cell<DIR>(g, l, k, i, j);
        const size_t q = IDX(i, j);
        out[q] = (T)(f.ty[q] - f.tp[q] * xs - f.tq[q] * xe);
    }
}

// FP64: the reference's Thomas recurrence (TRIDx_ser / TRIDy_ser,
// tridiagnal.F:338-398; periodic y: TRIDy_periodic, :59-325) in its own
// operation order, in two kernels.
//   k_thomas_rows (one thread per cell) computes every row's a, c, d
//   (etauv_solver.F:406-409, 504-507), with TRIDy_periodic's end-row
//   scaling, and stores what the recurrence needs: 1/a, c/a, d/a for a row
//   that is eliminated (a != 0 and not the first row), else 0, c, d.
//   k_thomas_lines (one thread per line) then walks the line: only the
//   dependent part, den = 1/a - c'(k-1), c' = (c/a)/den and
//   d' = (d/a - d'(k-1))/den, is on its critical path, and the loads of the
//   next block of rows are issued before the current block is worked.
// The results equal the one-pass recurrence bit for bit: the same IEEE
// operations on the same operands, in a translation unit compiled without
// contraction.  Scratch: tc = 1/a, tp = c/a then c', ty = d/a then d' then
// the first solution, tq = e' then the second solution (periodic).
template <typename T, int DIR, bool PER>
__global__ void __launch_bounds__(256) k_thomas_rows(Grid g, Fields<T> f, LinePart lp) {
    const int i = g.ib + blockIdx.x * blockDim.x + threadIdx.x;
    const int j = g.jb + blockIdx.y * blockDim.y + threadIdx.y;
    if (i > g.ie || j > g.je) return;
    const int k = DIR == 0 ? i - g.ib : j - g.jb;
    double a, c, d;
    tri_coef<T, DIR>(g, f, i, j, a, c, d);
    if (PER) {
        if (k == 0) {  // scaled by 1 + c_end, the c of the line's last row
            double a2, c2, d2;
            tri_coef<T, DIR>(g, f, DIR == 0 ? g.ie : i, DIR == 0 ? j : g.je, a2, c2, d2);
            c = c / (1 + c2);
            d = d / (1 + c2);
        }
        if (k == lp.L - 1) {  // scaled by 1 + a_beg, the a of the first row
            double a2, c2, d2;
            tri_coef<T, DIR>(g, f, DIR == 0 ? g.ib : i, DIR == 0 ? j : g.jb, a2, c2, d2);
            a = a / (1 + a2);
            d = d / (1 + a2);
        }
    }
    const size_t q = IDX(i, j);
    if (k > 0 && a != 0.0) {
        f.tc[q] = 1.0 / a;
        f.tp[q] = c / a;
        f.ty[q] = d / a;
    } else {
        f.tc[q] = 0.0;
        f.tp[q] = c;
        f.ty[q] = d;
    }
}

template <typename T, int DIR, bool PER>
__global__ void __launch_bounds__(32) k_thomas_lines(Grid g, Fields<T> f, LinePart lp) {
    constexpr int U = 8;  // rows per block of loads
    const int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= lp.nlines) return;
    const int L = lp.L;
    const size_t base = DIR == 0 ? IDX(g.ib, g.jb + l) : IDX(g.ib + l, g.jb);
    const size_t step = DIR == 0 ? 1 : (size_t)g.pitch;
    double a_beg = 0.0, c_end = 0.0, e_first = 0.0, e_last = 0.0, ea_last = 0.0;
    if (PER) {
        double a, c, d;
        int i, j;
        line_cell<DIR>(g, l, 0, i, j);
        tri_coef<T, DIR>(g, f, i, j, a, c, d);
        a_beg = a;
        line_cell<DIR>(g, l, L - 1, i, j);
        tri_coef<T, DIR>(g, f, i, j, a, c, d);
        c_end = c;
        // e = [1/(1+c_end), 0, ..., 0, -1/(1+a_beg)] (tridiagnal.F:207-215);
        // the last row eliminates e/a with its scaled a
        e_first = 1.0 / (1.0 + c_end);
        e_last = -1.0 / (1.0 + a_beg);
        ea_last = e_last / (a / (1 + a_beg));
    }
    double cra[U], cca[U], cda[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
        const size_t q = base + (size_t)u * step;
        cra[u] = u < L ? f.tc[q] : 0.0;
        cca[u] = u < L ? f.tp[q] : 0.0;
        cda[u] = u < L ? f.ty[q] : 0.0;
    }
    double cp = 0.0, dp = 0.0, ep = 0.0;
    for (int k0 = 0; k0 < L; k0 += U) {
        double nra[U], nca[U], nda[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int kk = k0 + U + u;
            const size_t q = base + (size_t)kk * step;
            nra[u] = kk < L ? f.tc[q] : 0.0;
            nca[u] = kk < L ? f.tp[q] : 0.0;
            nda[u] = kk < L ? f.ty[q] : 0.0;
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int k = k0 + u;
            if (k < L) {
                double c, d, e = 0.0;
                if (cra[u] != 0.0) {
                    const double den = cra[u] - cp;
                    c = cca[u] / den;
                    d = (cda[u] - dp) / den;
                    // e/a: 0/a is a zero with the sign of a (that of 1/a)
                    if (PER) e = ((k == L - 1 ? ea_last : fcopysign(0.0, cra[u])) - ep) / den;
                } else {
                    c = cca[u];
                    d = cda[u];
                    if (PER) e = k == L - 1 ? e_last : (k == 0 ? e_first : 0.0);
                }
                cp = c;
                dp = d;
                ep = e;
                const size_t q = base + (size_t)k * step;
                f.tp[q] = c;
                f.ty[q] = d;
                if (PER) f.tq[q] = e;
            }
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
            cra[u] = nra[u];
            cca[u] = nca[u];
            cda[u] = nda[u];
        }
    }
    // back substitution, blocks of U rows from the end; the first solution
    // into ty, the second into tq (periodic), else straight into U / V
    T *out = DIR == 0 ? f.U : f.V;
    double z1 = 0.0, z2 = 0.0;
    const int nblk = (L + U - 1) / U;
    double ccp[U], cdp[U], cep[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
        const int k = L - 1 - u;
        const size_t q = base + (size_t)(k >= 0 ? k : 0) * step;
        ccp[u] = k >= 0 ? f.tp[q] : 0.0;
        cdp[u] = k >= 0 ? f.ty[q] : 0.0;
        cep[u] = (PER && k >= 0) ? f.tq[q] : 0.0;
    }
    for (int b = 0; b < nblk; b++) {
        double ncp[U], ndp[U], nep[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int k = L - 1 - (b + 1) * U - u;
            const size_t q = base + (size_t)(k >= 0 ? k : 0) * step;
            ncp[u] = k >= 0 ? f.tp[q] : 0.0;
            ndp[u] = k >= 0 ? f.ty[q] : 0.0;
            nep[u] = (PER && k >= 0) ? f.tq[q] : 0.0;
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int k = L - 1 - b * U - u;
            if (k >= 0) {
                if (k == L - 1) {
                    z1 = cdp[u];
                    if (PER) z2 = cep[u];
                } else {
                    z1 = cdp[u] - ccp[u] * z1;
                    if (PER) z2 = cep[u] - ccp[u] * z2;
                }
                const size_t q = base + (size_t)k * step;
                if (PER) {
                    f.ty[q] = z1;
                    f.tq[q] = z2;
                } else {
                    out[q] = (T)z1;
                }
            }
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
            ccp[u] = ncp[u];
            cdp[u] = ndp[u];
            cep[u] = nep[u];
        }
    }
    if (PER) {
        const size_t q0 = base, q1 = base + (size_t)(L - 1) * step;
        const double beta = (c_end * f.ty[q0] - a_beg * f.ty[q1]) / (1.0 - (c_end * f.tq[q0] - a_beg * f.tq[q1]));
        for (int k = 0; k < L; k++) {
            const size_t q = base + (size_t)k * step;
            out[q] = (T)(f.ty[q] + beta * f.tq[q]);
        }
    }
}

// Mixed path: the tridiagonal matrices depend on Depth and MASK9 only, so
// their partitioned factorisation is computed (in double) when MASK9 has
// changed - never again once viscosity breaking has set MASK9 = 1 on the
// ring - and stored rounded to float.  Each stage then solves in float and
// refines once: x0 = S(d), r = d - T x0 with a compensated (float-pair)
// residual, x = x0 + S(r).  S is the partitioned substitution: per chunk of
// m rows a forward/backward sweep, a reduced system of two rows per chunk,
// and the interior recovery x_k = y_k - p_k x_s - q_k x_e.  For periodic y,
// S applies TRIDy_periodic's end-row scaling and Sherman-Morrison
// combination, whose result solves the cyclic system
// x0 + c0 x1 + a0 x(L-1) = d0, a(L-1) x(L-2) + x(L-1) + c(L-1) x0 = d(L-1)
// (tridiagnal.F:59-325); the residual uses that cyclic operator.
struct FacLine {
    float *lo, *di, *up, *cs, *ae, *x2, *tail;  // reduced rows; tail: c_end, a_beg, den_beta
};
__device__ __forceinline__ FacLine fac_line(float *base, const LinePart &lp, int l) {
    const int n = 2 * lp.P;
    float *b = base + (size_t)l * (size_t)(4 * n + 2 * lp.P + 3);
    FacLine f;
    f.lo = b;
    f.di = b + n;
    f.up = b + 2 * n;
    f.cs = b + 3 * n;
    f.ae = b + 3 * n + lp.P;
    f.x2 = b + 3 * n + 2 * lp.P;
    f.tail = b + 4 * n + 2 * lp.P;
    return f;
}

// normalised a, c and 1/tmp2 of one row, in double (no right-hand side)
template <typename T, int DIR>
__device__ __forceinline__ void tri_ac(const Grid &g, const Fields<T> &f, int i, int j, double &a, double &c,
                                       double &it) {
    const double mdf = g.min_depth_frc;
    const size_t id = IDX(i, j);
    const double dep = tmax((double)f.Depth[id], mdf);
    const double depl = tmax((double)f.Depth[DIR == 0 ? IDX(i - 1, j) : IDX(i, j - 1)], mdf);
    const double depr = tmax((double)f.Depth[DIR == 0 ? IDX(i + 1, j) : IDX(i, j + 1)], mdf);
    const double gm = g.gamma1 * (double)f.MASK9[id];
    const double tmp1 = gm * dep * (g.cA[DIR] * dep + g.cB[DIR] * depl);
    const double tmp2 = 1.0 + gm * g.cC[DIR] * dep * dep;
    const double tmp3 = gm * dep * (g.cA[DIR] * dep + g.cB[DIR] * depr);
    it = 1.0 / tmp2;
    a = tmp1 * it;
    c = tmp3 * it;
}

// a, c of row k with the periodic end-row scaling (tridiagnal.F:168-173)
template <typename T, int DIR, bool PER>
__device__ __forceinline__ void tri_ac_row(const Grid &g, const Fields<T> &f, const LinePart &lp, int l, int k,
                                           double &a, double &c, double &it) {
    int i, j;
    line_cell<DIR>(g, l, k, i, j);
    tri_ac<T, DIR>(g, f, i, j, a, c, it);
    if (PER && (k == 0 || k == lp.L - 1)) {
        double a2, c2, it2;
        int i2, j2;
        line_cell<DIR>(g, l, k == 0 ? lp.L - 1 : 0, i2, j2);
        tri_ac<T, DIR>(g, f, i2, j2, a2, c2, it2);
        if (k == 0) c = c / (1 + c2);   // c_end
        else a = a / (1 + a2);           // a_beg
    }
}

__device__ __forceinline__ void split2(double v, float &hi, float &lo) {
    hi = (float)v;
    lo = (float)(v - (double)hi);
}

template <typename T, int DIR, bool PER>
__device__ __forceinline__ void fac_a_body(const Grid &g, const Fields<T> &f, const LinePart &lp, int t) {
    if (t >= lp.nlines * lp.P) return;
    int l, ch;
    chunk_of<DIR>(lp, t, l, ch);
    const int s = ch * lp.m;
    const int e = (ch == lp.P - 1) ? lp.L - 1 : s + lp.m - 1;
    float *it_ = f.fac_it[DIR], *A_ = f.fac_A[DIR], *lr_ = f.fac_lr[DIR], *cp_ = f.fac_cp[DIR];
    float *p_ = f.fac_p[DIR], *q_ = f.fac_q[DIR];
    // the unscaled normalised coefficients of every row, for the residual
    for (int k = s; k <= e; k++) {
        double a, c, it;
        int i, j;
        line_cell<DIR>(g, l, k, i, j);
        tri_ac<T, DIR>(g, f, i, j, a, c, it);
        if (!PER && k == 0) a = 0.0;
        if (!PER && k == lp.L - 1) c = 0.0;
        const size_t q = IDX(i, j);
        split2(a, f.fac_ah[DIR][q], f.fac_al[DIR][q]);
        split2(c, f.fac_ch[DIR][q], f.fac_cl[DIR][q]);
        it_[q] = (float)it;
    }
    double as, cs, its, ae, ce, ite;
    tri_ac_row<T, DIR, PER>(g, f, lp, l, s, as, cs, its);
    tri_ac_row<T, DIR, PER>(g, f, lp, l, e, ae, ce, ite);
    int i, j;
    line_cell<DIR>(g, l, s, i, j);
    A_[IDX(i, j)] = 1.0f;
    line_cell<DIR>(g, l, e, i, j);
    A_[IDX(i, j)] = 1.0f;
    if (s == 0) as = 0.0;
    if (e == lp.L - 1) ce = 0.0;
    double lo_s, di_s, up_s, lo_e, di_e, up_e;
    if (e - s >= 2) {
        double cp = 0.0, pp = 0.0, qp = 0.0;
        double *pbuf = f.sw_p[DIR], *qbuf = f.sw_q[DIR], *cbuf = f.sw_c[DIR];  // sweep scratch of this direction
        for (int k = s + 1; k <= e - 1; k++) {
            double a, c, it;
            tri_ac_row<T, DIR, PER>(g, f, lp, l, k, a, c, it);
            const double lower = (k > s + 1) ? a : 0.0;
            const double r = 1.0 / (1.0 - lower * cp);
            const double upper = (k < e - 1) ? c : 0.0;
            cp = upper * r;
            pp = ((k == s + 1 ? a : 0.0) - lower * pp) * r;
            qp = ((k == e - 1 ? c : 0.0) - lower * qp) * r;
            line_cell<DIR>(g, l, k, i, j);
            const size_t q = IDX(i, j);
            A_[q] = (float)r;
            lr_[q] = (float)(lower * r);
            cp_[q] = (float)cp;
            cbuf[q] = cp;
            pbuf[q] = pp;
            qbuf[q] = qp;
        }
        double pn = 0.0, qn = 0.0, p1 = 0.0, q1 = 0.0, pl = 0.0, ql = 0.0;
        for (int k = e - 1; k >= s + 1; k--) {
            line_cell<DIR>(g, l, k, i, j);
            const size_t q = IDX(i, j);
            const double cpk = cbuf[q];
            const double pk = pbuf[q] - cpk * pn, qk = qbuf[q] - cpk * qn;
            p_[q] = (float)pk;
            q_[q] = (float)qk;
            pn = pk;
            qn = qk;
            if (k == e - 1) {
                pl = pk;
                ql = qk;
            }
            if (k == s + 1) {
                p1 = pk;
                q1 = qk;
            }
        }
        lo_s = as;
        di_s = 1.0 - cs * p1;
        up_s = -cs * q1;
        lo_e = -ae * pl;
        di_e = 1.0 - ae * ql;
        up_e = ce;
    } else {
        lo_s = as;
        di_s = 1.0;
        up_s = cs;
        lo_e = ae;
        di_e = 1.0;
        up_e = ce;
    }
    // reduced rows to the double scratch; k_fac_b factors them
    double *red = f.red + lp.red0 + ((size_t)l * 2 * lp.P + 2 * ch) * 6;
    red[0] = lo_s;
    red[1] = di_s;
    red[2] = up_s;
    red[6] = lo_e;
    red[7] = di_e;
    red[8] = up_e;
    FacLine fl = fac_line(f.fac_red[DIR], lp, l);
    fl.cs[ch] = (e - s >= 2) ? (float)cs : 0.0f;
    fl.ae[ch] = (e - s >= 2) ? (float)ae : 0.0f;
}

template <typename T, int DIR, bool PER>
__global__ void __launch_bounds__(128) k_fac_a(Grid g, Fields<T> f, LinePart lp) {
    if (!*f.m9_dirty) return;
    fac_a_body<T, DIR, PER>(g, f, lp, blockIdx.x * blockDim.x + threadIdx.x);
}

template <typename T, int DIR, bool PER>
__device__ __forceinline__ void fac_b_body(const Grid &g, const Fields<T> &f, const LinePart &lp, int l) {
    if (l >= lp.nlines) return;
    const int n = 2 * lp.P;
    double *red = f.red + lp.red0 + (size_t)l * n * 6;
    FacLine fl = fac_line(f.fac_red[DIR], lp, l);
    double cpr = 0.0;
    for (int k = 0; k < n; k++) {
        const double lo = (k > 0) ? red[k * 6 + 0] : 0.0;
        const double up = (k < n - 1) ? red[k * 6 + 2] : 0.0;
        const double id = 1.0 / (red[k * 6 + 1] - lo * cpr);
        cpr = up * id;
        fl.lo[k] = (float)lo;       // the reduced rows, solved per stage by
        fl.di[k] = (float)red[k * 6 + 1];  // parallel cyclic reduction
        fl.up[k] = (float)up;
        red[k * 6 + 3] = lo;   // double factors for the periodic solve below
        red[k * 6 + 4] = id;
        red[k * 6 + 5] = cpr;
    }
    if (PER) {
        // the second periodic solution (right-hand side e of TRIDy_periodic,
        // tridiagnal.F:207-215) and the constant denominator of beta
        double a, c, it;
        int i, j;
        line_cell<DIR>(g, l, 0, i, j);
        tri_ac<T, DIR>(g, f, i, j, a, c, it);
        const double a_beg = a;
        line_cell<DIR>(g, l, lp.L - 1, i, j);
        tri_ac<T, DIR>(g, f, i, j, a, c, it);
        const double c_end = c;
        double z = 0.0;
        for (int k = 0; k < n; k++) {
            const double rhs = k == 0 ? 1.0 / (1.0 + c_end) : (k == n - 1 ? -1.0 / (1.0 + a_beg) : 0.0);
            z = (rhs - red[k * 6 + 3] * z) * red[k * 6 + 4];
            red[k * 6 + 0] = z;
        }
        double x = 0.0, x0 = 0.0, xl = 0.0;
        for (int k = n - 1; k >= 0; k--) {
            x = red[k * 6 + 0] - red[k * 6 + 5] * x;
            fl.x2[k] = (float)x;
            if (k == n - 1) xl = x;
            if (k == 0) x0 = x;
        }
        fl.tail[0] = (float)c_end;
        fl.tail[1] = (float)a_beg;
        fl.tail[2] = (float)(1.0 - (c_end * x0 - a_beg * xl));
    }
}

template <typename T, int DIR, bool PER>
__global__ void __launch_bounds__(128) k_fac_b(Grid g, Fields<T> f, LinePart lp) {
    if (!*f.m9_dirty) return;
    fac_b_body<T, DIR, PER>(g, f, lp, blockIdx.x * blockDim.x + threadIdx.x);
}

// both directions in one launch each: blocks [0, nbx) factor x, the rest y
template <typename T, bool PERY>
__global__ void __launch_bounds__(128) k_fac_a_xy(Grid g, Fields<T> f, LinePart px, LinePart py, int nbx) {
    if (!*f.m9_dirty) return;
    if ((int)blockIdx.x < nbx) fac_a_body<T, 0, false>(g, f, px, blockIdx.x * blockDim.x + threadIdx.x);
    else fac_a_body<T, 1, PERY>(g, f, py, (blockIdx.x - nbx) * blockDim.x + threadIdx.x);
}
template <typename T, bool PERY>
__global__ void __launch_bounds__(128) k_fac_b_xy(Grid g, Fields<T> f, LinePart px, LinePart py, int nbx) {
    if (!*f.m9_dirty) return;
    if ((int)blockIdx.x < nbx) fac_b_body<T, 0, false>(g, f, px, blockIdx.x * blockDim.x + threadIdx.x);
    else fac_b_body<T, 1, PERY>(g, f, py, (blockIdx.x - nbx) * blockDim.x + threadIdx.x);
}

static __global__ void k_fac_clear(int *dirty) { *dirty = 0; }

// compensated r = d - (a x(k-1) + x(k) + c x(k+1)) with a = ah + al, c = ch + cl
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}
__device__ __forceinline__ void two_prod(float a, float b, float &p, float &e) {
    p = a * b;
    e = fmaf(a, b, -p);
}
__device__ __forceinline__ float residual(float d, float x, float xm, float xp, float ah, float al, float ch,
                                          float cl) {
    float t, e1, u, e2, v, e3, t2, e4, t3, e5;
    two_sum(d, -x, t, e1);
    two_prod(ah, xm, u, e2);
    two_prod(ch, xp, v, e3);
    two_sum(t, -u, t2, e4);
    two_sum(t2, -v, t3, e5);
    return t3 + ((((e1 + e4) + e5) - e2) - e3 - al * xm - cl * xp);
}

// Parallel cyclic reduction of n reduced rows lo x(k-1) + di x(k) +
// up x(k+1) = r in shared memory by the whole block: log2(n) steps, each row
// eliminating its neighbours at distance s; the solution replaces r.
// Buffers: lo, di, up, r and their doubles lo2, di2, up2, r2 (n floats each).
__device__ __forceinline__ void pcr_solve(float *lo, float *di, float *up, float *r, float *lo2, float *di2,
                                          float *up2, float *r2, int n) {
    for (int st = 1; st < n; st <<= 1) {
        for (int k = threadIdx.x; k < n; k += blockDim.x) {
            const int km = k - st, kp = k + st;
            float a = 0.0f, b = 0.0f, nlo = 0.0f, nup = 0.0f;
            float nd = di[k], nr = r[k];
            if (km >= 0) {
                a = -lo[k] / di[km];
                nlo = a * lo[km];
                nd += a * up[km];
                nr += a * r[km];
            }
            if (kp < n) {
                b = -up[k] / di[kp];
                nup = b * up[kp];
                nd += b * lo[kp];
                nr += b * r[kp];
            }
            lo2[k] = nlo;
            di2[k] = nd;
            up2[k] = nup;
            r2[k] = nr;
        }
        __syncthreads();
        float *t;
        t = lo; lo = lo2; lo2 = t;
        t = di; di = di2; di2 = t;
        t = up; up = up2; up2 = t;
        t = r; r = r2; r2 = t;
    }
    // after the last swap the current buffers may be the doubles: copy the
    // solution into both
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        const float x = r[k] / di[k];
        r[k] = x;
        r2[k] = x;
    }
    __syncthreads();
}

// y lines (and the periodic direction): per-chunk kernels, coalesced across
// neighbouring lines.  PASS 0 solves d = rhs/tmp2, PASS 1 the residual.
// per-stage reduced right-hand sides: pass 0 at the start of the scratch,
// pass 1 right after it
template <int PASS> __device__ __forceinline__ float *red_rhs(double *red, const LinePart &lp) {
    return (float *)red + (PASS == 0 ? 0 : (size_t)lp.nlines * 2 * lp.P);
}

// M > 0: chunks of exactly M rows are walked in registers (all loads first,
// the sweep values stored once); other chunks, and M = 0, walk the loop.
// Both do the same operations in the same order.
template <typename T, int DIR, bool PER, int PASS, int M>
__global__ void __launch_bounds__(128) k_sol_a(Grid g, Fields<T> f, LinePart lp) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= lp.nlines * lp.P) return;
    int l, ch;
    chunk_of<DIR>(lp, t, l, ch);
    const int s = ch * lp.m;
    const int e = (ch == lp.P - 1) ? lp.L - 1 : s + lp.m - 1;
    const T *rhs = DIR == 0 ? f.rhs_x : f.rhs_y;
    const float *it_ = f.fac_it[DIR], *A_ = f.fac_A[DIR], *lr_ = f.fac_lr[DIR], *cp_ = f.fac_cp[DIR];
    float *ys = (float *)f.ty;   // y of this pass
    const float *rr = (const float *)f.tq;  // residual (PASS 1)
    FacLine fl = fac_line(f.fac_red[DIR], lp, l);
    float sc0 = 1.0f, sc1 = 1.0f;
    if (PER) {
        sc0 = 1.0f / (1.0f + fl.tail[0]);  // row 0: d / (1 + c_end)
        sc1 = 1.0f / (1.0f + fl.tail[1]);  // row L-1: d / (1 + a_beg)
    }
    auto dval = [&](int k, size_t q) {
        float d = PASS == 0 ? (float)rhs[q] * it_[q] : rr[q];
        if (PER && k == 0) d *= sc0;
        if (PER && k == lp.L - 1) d *= sc1;
        return d;
    };
    int i, j;
    line_cell<DIR>(g, l, s, i, j);
    const float ds = dval(s, IDX(i, j));
    line_cell<DIR>(g, l, e, i, j);
    const float de = dval(e, IDX(i, j));
    float rs = ds, re = de;
    if constexpr (M > 2) {
        if (e - s + 1 == M) {
            const size_t stride = DIR == 0 ? 1 : (size_t)g.pitch;
            line_cell<DIR>(g, l, s, i, j);
            const size_t q0 = IDX(i, j);
            float dv[M], av[M], lv[M], cv[M], yv[M];
#pragma unroll
            for (int k = 1; k < M - 1; k++) {
                const size_t q = q0 + (size_t)k * stride;
                dv[k] = dval(s + k, q);
                av[k] = A_[q];
                lv[k] = lr_[q];
                cv[k] = cp_[q];
            }
            float yp = 0.0f;
#pragma unroll
            for (int k = 1; k < M - 1; k++) {
                yp = dv[k] * av[k] - lv[k] * yp;
                yv[k] = yp;
            }
            float yn = 0.0f;
#pragma unroll
            for (int k = M - 2; k >= 1; k--) {
                yn = yv[k] - cv[k] * yn;
                yv[k] = yn;
            }
#pragma unroll
            for (int k = 1; k < M - 1; k++) ys[q0 + (size_t)k * stride] = yv[k];
            rs = ds - fl.cs[ch] * yv[1];
            re = de - fl.ae[ch] * yv[M - 2];
            float *red = red_rhs<PASS>(f.red, lp) + ((size_t)l * 2 * lp.P + 2 * ch);
            red[0] = rs;
            red[1] = re;
            return;
        }
    }
    if (e - s >= 2) {
        float yp = 0.0f;
        for (int k = s + 1; k <= e - 1; k++) {
            line_cell<DIR>(g, l, k, i, j);
            const size_t q = IDX(i, j);
            yp = dval(k, q) * A_[q] - lr_[q] * yp;
            ys[q] = yp;
        }
        float yn = 0.0f, y1 = 0.0f, yl = 0.0f;
        for (int k = e - 1; k >= s + 1; k--) {
            line_cell<DIR>(g, l, k, i, j);
            const size_t q = IDX(i, j);
            const float yk = ys[q] - cp_[q] * yn;
            ys[q] = yk;
            yn = yk;
            if (k == e - 1) yl = yk;
            if (k == s + 1) y1 = yk;
        }
        rs = ds - fl.cs[ch] * y1;
        re = de - fl.ae[ch] * yl;
    }
    float *red = red_rhs<PASS>(f.red, lp) + ((size_t)l * 2 * lp.P + 2 * ch);
    red[0] = rs;
    red[1] = re;
}

template <typename T, int DIR, bool PER, int PASS>
__global__ void __launch_bounds__(512) k_sol_b(Grid g, Fields<T> f, LinePart lp) {
    extern __shared__ float shr[];
    const int l = blockIdx.x;
    const int n = 2 * lp.P;
    float *red = red_rhs<PASS>(f.red, lp) + (size_t)l * n;
    FacLine fl = fac_line(f.fac_red[DIR], lp, l);
    float *lo = shr, *di = shr + n, *up = shr + 2 * n, *r = shr + 3 * n;
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        lo[k] = fl.lo[k];
        di[k] = fl.di[k];
        up[k] = fl.up[k];
        r[k] = red[k];
    }
    __syncthreads();
    pcr_solve(lo, di, up, r, shr + 4 * n, shr + 5 * n, shr + 6 * n, shr + 7 * n, n);
    float beta = 0.0f;
    if (PER) beta = (fl.tail[0] * r[0] - fl.tail[1] * r[n - 1]) / fl.tail[2];
    for (int k = threadIdx.x; k < n; k += blockDim.x) red[k] = PER ? r[k] + beta * fl.x2[k] : r[k];
}

// PASS 0: x0 -> tp scratch; PASS 1: out = x0 + correction.  M > 0: chunks
// of exactly M rows with all loads first (as k_sol_a).
template <typename T, int DIR, int PASS, int M>
__global__ void __launch_bounds__(128) k_sol_c(Grid g, Fields<T> f, LinePart lp) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= lp.nlines * lp.P) return;
    int l, ch;
    chunk_of<DIR>(lp, t, l, ch);
    const int s = ch * lp.m;
    const int e = (ch == lp.P - 1) ? lp.L - 1 : s + lp.m - 1;
    const float *red = red_rhs<PASS>(f.red, lp) + ((size_t)l * 2 * lp.P + 2 * ch);
    const float xs = red[0], xe = red[1];
    const float *p_ = f.fac_p[DIR], *q_ = f.fac_q[DIR];
    const float *ys = (const float *)f.ty;
    float *x0 = (float *)f.tp;
    T *out = DIR == 0 ? f.U : f.V;
    if constexpr (M > 2) {
        if (e - s + 1 == M) {
            const size_t stride = DIR == 0 ? 1 : (size_t)g.pitch;
            int i, j;
            line_cell<DIR>(g, l, s, i, j);
            const size_t q0 = IDX(i, j);
            float xv[M], x0v[M];
#pragma unroll
            for (int k = 0; k < M; k++) {
                const size_t q = q0 + (size_t)k * stride;
                xv[k] = (k == 0) ? xs : (k == M - 1) ? xe : ys[q] - p_[q] * xs - q_[q] * xe;
                if (PASS == 1) x0v[k] = x0[q];
            }
#pragma unroll
            for (int k = 0; k < M; k++) {
                const size_t q = q0 + (size_t)k * stride;
                if (PASS == 0) x0[q] = xv[k];
                else out[q] = (T)(x0v[k] + xv[k]);
            }
            return;
        }
    }
    for (int k = s; k <= e; k++) {
        int i, j;
        line_cell<DIR>(g, l, k, i, j);
        const size_t q = IDX(i, j);
        const float x = (k == s) ? xs : (k == e) ? xe : ys[q] - p_[q] * xs - q_[q] * xe;
        if (PASS == 0) x0[q] = x;
        else out[q] = (T)(x0[q] + x);
    }
}

// compensated residual of the first solve on every interior cell
template <typename T, int DIR, bool PER>
__global__ void __launch_bounds__(256) k_resid(Grid g, Fields<T> f, LinePart lp) {
    const int i = g.ib + blockIdx.x * blockDim.x + threadIdx.x;
    const int j = g.jb + blockIdx.y * blockDim.y + threadIdx.y;
    if (i > g.ie || j > g.je) return;
    const size_t q = IDX(i, j);
    const int k = DIR == 0 ? i - g.ib : j - g.jb;
    const size_t st = DIR == 0 ? 1 : (size_t)g.pitch;
    const float *x0 = (const float *)f.tp;
    const T *rhs = DIR == 0 ? f.rhs_x : f.rhs_y;
    const float d = (float)rhs[q] * f.fac_it[DIR][q];
    // neighbours along the line; the cyclic ends wrap in periodic y
    float xm = 0.0f, xp = 0.0f;
    if (k > 0) xm = x0[q - st];
    else if (PER) xm = x0[q + (size_t)(lp.L - 1) * st];
    if (k < lp.L - 1) xp = x0[q + st];
    else if (PER) xp = x0[q - (size_t)(lp.L - 1) * st];
    ((float *)f.tq)[q] = residual(d, x0[q], xm, xp, f.fac_ah[DIR][q], f.fac_al[DIR][q], f.fac_ch[DIR][q],
                                  f.fac_cl[DIR][q]);
}

// x lines, one block per line, everything unit-stride: load d, solve, form
// the compensated residual, solve again and write x0 + correction.  The
// arrays that a thread walks along its own chunk are stored with one pad
// float after every 16 (index k + k/16), so that the 32 chunks a warp walks
// at once fall into different shared-memory banks.
__host__ __device__ __forceinline__ int lsx_pad(int k) { return k + (k >> 4); }
__host__ __device__ __forceinline__ size_t lsx_smem_floats(int L, int P) {
    return (size_t)6 * (lsx_pad(L) + 1) + (size_t)L + 16 * (size_t)P;
}

// KPT > 0: lines of at most 256 x KPT cells; every global value a thread
// needs later (the reconstruction's p, q and the residual's a, c pairs of
// its cells k = tid + 256 j, the reduced rows and the chunk's spike ends)
// is loaded into registers at the start, together with the staging loads,
// so that the block waits for global memory once instead of once per phase.
// KPT = 0: any length, loads where they are used.
template <typename T, int KPT>
__global__ void __launch_bounds__(256, KPT > 0 ? 3 : 1) k_linesolve_x(Grid g, Fields<T> f, LinePart lp, int clear_dirty) {
    extern __shared__ float shf[];
    const int l = blockIdx.x;
    // the factorisation of this stage is complete: the MASK9 change flag
    // can be reset for UPDATE_MASK to set again
    if (clear_dirty && l == 0 && threadIdx.x == 0) *f.m9_dirty = 0;
    const int L = lp.L, P = lp.P, m = lp.m;
    const int LP = lsx_pad(L) + 1;
    float *d = shf;            // right-hand side, then residual (padded)
    float *y = shf + LP;       // sweep values (padded)
    float *A = shf + 2 * LP;   // sweep constants, staged with unit-stride loads (padded)
    float *LR = shf + 3 * LP;
    float *CP = shf + 4 * LP;
    float *dn = shf + 5 * LP;  // the normalised right-hand side, kept for the residual (padded)
    float *x0 = shf + 6 * LP;  // L  first solution (unpadded)
    float *rr = x0 + L;        // 2P reduced right-hand sides / solution
    float *pb = rr + 2 * P;    // 7 x 2P PCR buffers
    const int j = g.jb + l;
    const size_t row = (size_t)j * g.pitch + g.ib;
    const T *rhs = f.rhs_x + row;
    const float *IT = f.fac_it[0] + row, *Pp = f.fac_p[0] + row, *Qq = f.fac_q[0] + row;
    const float *AH = f.fac_ah[0] + row, *AL = f.fac_al[0] + row;
    const float *CH = f.fac_ch[0] + row, *CL = f.fac_cl[0] + row;
    FacLine fl = fac_line(f.fac_red[0], lp, l);
    const int ch = threadIdx.x;
    const int s = ch * m;
    const int e = (ch == P - 1) ? L - 1 : s + m - 1;
    const int n = 2 * P;
    constexpr int KR = KPT > 0 ? KPT : 1;
    float rP[KR], rQ[KR], rAH[KR], rAL[KR], rCH[KR], rCL[KR];
    float lo_r = 0.0f, di_r = 0.0f, up_r = 0.0f, cs_r = 0.0f, ae_r = 0.0f;
    if constexpr (KPT > 0) {
#pragma unroll
        for (int q = 0; q < KPT; q++) {
            const int k = threadIdx.x + q * 256;
            if (k < L) {
                rP[q] = Pp[k];
                rQ[q] = Qq[k];
                rAH[q] = AH[k];
                rAL[q] = AL[k];
                rCH[q] = CH[k];
                rCL[q] = CL[k];
            }
        }
        if ((int)threadIdx.x < n) {
            lo_r = fl.lo[threadIdx.x];
            di_r = fl.di[threadIdx.x];
            up_r = fl.up[threadIdx.x];
        }
        if (ch < P) {
            cs_r = fl.cs[ch];
            ae_r = fl.ae[ch];
        }
    }
    for (int k = threadIdx.x; k < L; k += blockDim.x) {
        const int q = lsx_pad(k);
        const float dv = (float)rhs[k] * IT[k];
        d[q] = dv;
        dn[q] = dv;
        A[q] = f.fac_A[0][row + k];
        LR[q] = f.fac_lr[0][row + k];
        CP[q] = f.fac_cp[0][row + k];
    }
    __syncthreads();
    for (int pass = 0; pass < 2; pass++) {
        // chunk forward/backward sweeps
        if (ch < P) {
            float rs = d[lsx_pad(s)], re = d[lsx_pad(e)];
            if (e - s >= 2) {
                float yp = 0.0f;
                for (int k = s + 1; k <= e - 1; k++) {
                    const int q = lsx_pad(k);
                    yp = d[q] * A[q] - LR[q] * yp;
                    y[q] = yp;
                }
                float yn = 0.0f;
                for (int k = e - 1; k >= s + 1; k--) {
                    const int q = lsx_pad(k);
                    yn = y[q] - CP[q] * yn;
                    y[q] = yn;
                }
                rs = rs - (KPT > 0 ? cs_r : fl.cs[ch]) * y[lsx_pad(s + 1)];
                re = re - (KPT > 0 ? ae_r : fl.ae[ch]) * y[lsx_pad(e - 1)];
            }
            rr[2 * ch] = rs;
            rr[2 * ch + 1] = re;
        }
        if constexpr (KPT > 0) {
            if ((int)threadIdx.x < n) {
                pb[threadIdx.x] = lo_r;
                pb[n + threadIdx.x] = di_r;
                pb[2 * n + threadIdx.x] = up_r;
            }
        } else {
            for (int k = threadIdx.x; k < n; k += blockDim.x) {
                pb[k] = fl.lo[k];
                pb[n + k] = fl.di[k];
                pb[2 * n + k] = fl.up[k];
            }
        }
        __syncthreads();
        pcr_solve(pb, pb + n, pb + 2 * n, rr, pb + 3 * n, pb + 4 * n, pb + 5 * n, pb + 6 * n, n);
        auto recon = [&](int k, float p_, float q_) {
            const int c = min(lp.lgm >= 0 ? k >> lp.lgm : k / m, P - 1);
            const int cs = c * m, ce = (c == P - 1) ? L - 1 : cs + m - 1;
            const float x = (k == cs) ? rr[2 * c] : (k == ce) ? rr[2 * c + 1] : y[lsx_pad(k)] - p_ * rr[2 * c] - q_ * rr[2 * c + 1];
            if (pass == 0) x0[k] = x;
            else f.U[row + k] = (T)(x0[k] + x);
        };
        if constexpr (KPT > 0) {
#pragma unroll
            for (int q = 0; q < KPT; q++) {
                const int k = threadIdx.x + q * 256;
                if (k < L) recon(k, rP[q], rQ[q]);
            }
        } else {
            for (int k = threadIdx.x; k < L; k += blockDim.x) recon(k, Pp[k], Qq[k]);
        }
        __syncthreads();
        if (pass == 0) {
            auto resid = [&](int k, float ah, float al, float chv, float cl) {
                const float xm = k > 0 ? x0[k - 1] : 0.0f, xp = k < L - 1 ? x0[k + 1] : 0.0f;
                const int q = lsx_pad(k);
                d[q] = residual(dn[q], x0[k], xm, xp, ah, al, chv, cl);
            };
            if constexpr (KPT > 0) {
#pragma unroll
                for (int q = 0; q < KPT; q++) {
                    const int k = threadIdx.x + q * 256;
                    if (k < L) resid(k, rAH[q], rAL[q], rCH[q], rCL[q]);
                }
            } else {
                for (int k = threadIdx.x; k < L; k += blockDim.x) resid(k, AH[k], AL[k], CH[k], CL[k]);
            }
            __syncthreads();
        }
    }
}

// ---------------------------------------------------------------------------
// GET_Eta_U_V_HU_HV tail (etauv_solver.F:558-600): dry zeroing, HU/HV and
// the Froude cap, with the MASK of the start of the stage.
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ void post_cell(const Grid &g, const Fields<T> &f, int i, int j) {
    const size_t id = IDX(i, j);
    const T mdf = GC(min_depth_frc);
    const bool interior = !(i < g.ib || i > g.ie || j < g.jb || j > g.je);
    if (interior) {
        if (!g.dispersion) {
            const T Hm = tmax(ro(f.H + (id)), mdf);
            f.U[id] = f.Ubar[id] / Hm;
            f.V[id] = f.Vbar[id] / Hm;
        }
        if (ro(f.MASK + (id)) < 1) {
            f.Ubar[id] = (T)0;
            f.Vbar[id] = (T)0;
            f.U[id] = (T)0;
            f.V[id] = (T)0;
            f.HU[id] = (T)0;
            f.HV[id] = (T)0;
        } else {
            const T Hm = tmax(ro(f.H + (id)), mdf);
            const T u = f.U[id], v = f.V[id];
            f.HU[id] = Hm * u;
            f.HV[id] = Hm * v;
            const T Utotal = fsqrt(u * u + v * v);
            const T Fr = fsqrt((T)GRAV * Hm);
            if (Utotal / Fr > GC(froude_cap)) {
                const T th = fatan2(v, u);
                const T un = GC(froude_cap) * Fr * fcos(th);
                const T vn = GC(froude_cap) * Fr * fsin(th);
                f.U[id] = un;
                f.V[id] = vn;
                f.HU[id] = un * Hm;
                f.HV[id] = vn * Hm;
            }
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(256) k_post(Grid g, Fields<T> f) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= g.Mloc || j >= g.Nloc) return;
    post_cell(g, f, i, j);
}

// Ubar = HU, Vbar = HV on every cell when DISPERSION is off (etauv_solver.F:596-600)
template <typename T>
__global__ void k_nodisp_copy(Grid g, Fields<T> f) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= g.Mloc || j >= g.Nloc) return;
    const size_t id = IDX(i, j);
    f.Ubar[id] = f.HU[id];
    f.Vbar[id] = f.HV[id];
}

// ---------------------------------------------------------------------------
// UPDATE_MASK (masks.F:51-205): MASK (Jacobi into MASKn), the Depthx/
// Depthy reset at old-dry cells, MASK9.  Launched over (Mloc+1) x (Nloc+1)
// so that every face has a thread.
// ---------------------------------------------------------------------------
// The sign of eta + h, with h the Depth as given in double (the FP64
// build's own Depth, the mixed build's double copy of it): +1 for
// eta > -h, -1 for eta < -h, 0 for equality, as the double comparisons of
// masks.F:107, 129 decide.  The mixed build decides in float where the
// float sum's margin exceeds its rounding (about 2 ulps of the larger term,
// plus the rounding of the stored float Depth), which gives the same sign,
// and evaluates the rest in double: FP64 instructions run only at cells
// within a few ulps of the threshold.
__device__ __forceinline__ int wet_test(double eta, double hf, const double *) {
    return eta > -hf ? 1 : (eta < -hf ? -1 : 0);
}
// the double comparison, out of line so that the float path of the callers
// keeps its registers
static __device__ __noinline__ int wet_test_double(float eta, const double *hdp) {
    const double e = (double)eta, hd = *hdp;
    return e > -hd ? 1 : (e < -hd ? -1 : 0);
}
__device__ __forceinline__ int wet_test(float eta, float hf, const double *hdp) {
    const float s = eta + hf;
    const float tol = 4.0e-7f * fmaxf(fabsf(eta), fabsf(hf)) + 1.0e-30f;
    if (s > tol) return 1;
    if (s < -tol) return -1;
    return wet_test_double(eta, hdp);  // the double depth only here
}

template <typename T>
__device__ __forceinline__ bool in_mask_range(const Grid &g, int a, int b) {
    return a >= g.ib - 2 && a <= g.ie + 2 && b >= g.jb - 2 && b <= g.je + 2;
}
template <typename T>
__device__ __forceinline__ int new_mask(const Grid &g, const Fields<T> &f, int a, int b) {
    const size_t q = IDX(a, b);
    const int m = ro(f.MASK + (q));
    if (!in_mask_range<T>(g, a, b) || ro(f.MASK_STRUC + (q)) != 1) return m;
    // total-depth tests (masks.F:107, 129) of eta against Depth as given, in
    // double (wet_test)
    const T eta = ro(f.Eta + (q));
    const int side = wet_test(eta, ro(f.Depth + (q)), f.DepthD + q);
    if (m < 1) {
        int r = m;
        if (side > 0) r = 1;
        if (ro(f.MASK + (IDX(a - 1, b))) == 1 && ro(f.Eta + (IDX(a - 1, b))) > eta) r = 1;
        if (ro(f.MASK + (IDX(a + 1, b))) == 1 && ro(f.Eta + (IDX(a + 1, b))) > eta) r = 1;
        if (ro(f.MASK + (IDX(a, b - 1))) == 1 && ro(f.Eta + (IDX(a, b - 1))) > eta) r = 1;
        if (ro(f.MASK + (IDX(a, b + 1))) == 1 && ro(f.Eta + (IDX(a, b + 1))) > eta) r = 1;
        return r;
    }
    return (side < 0) ? 0 : m;
}

// one thread of UPDATE_MASK at (i, j) in 0..Mloc x 0..Nloc
template <typename T>
__device__ __forceinline__ void mask_cell(const Grid &g, const Fields<T> &f, int i, int j) {
    // Depthx at x-face i of row j
    if (j < g.Nloc && j >= g.jb - 2 && j <= g.je + 2) {
        const bool rin = (i >= g.ib - 2 && i <= g.ie + 2);
        const bool lin = (i - 1 >= g.ib - 2 && i - 1 <= g.ie + 2);
        if (rin && ro(f.MASK + (IDX(i, j))) < 1) f.Depthx[IDX(i, j)] = ro(f.Depth + (IDX(i - 1, j)));
        else if (lin && ro(f.MASK + (IDX(i - 1, j))) < 1) f.Depthx[IDX(i, j)] = ro(f.Depth + (IDX(i, j)));
    }
    // Depthy at y-face j of column i
    if (i < g.Mloc && i >= g.ib - 2 && i <= g.ie + 2) {
        const bool tin = (j >= g.jb - 2 && j <= g.je + 2);
        const bool bin = (j - 1 >= g.jb - 2 && j - 1 <= g.je + 2);
        if (tin && ro(f.MASK + (IDX(i, j))) < 1) f.Depthy[IDX(i, j)] = ro(f.Depth + (IDX(i, j - 1)));
        else if (bin && ro(f.MASK + (IDX(i, j - 1))) < 1) f.Depthy[IDX(i, j)] = ro(f.Depth + (IDX(i, j)));
    }
    if (i >= g.Mloc || j >= g.Nloc) return;
    const size_t id = IDX(i, j);
    f.MASKn[id] = (uint8_t)new_mask(g, f, i, j);
    // MASK9 on Ibeg-1..Iend+1 x Jbeg-1..Jend+1; 0 elsewhere (never written
    // in the reference, whose temporary is fresh memory)
    uint8_t m9 = 0;
    if (i >= g.ib - 1 && i <= g.ie + 1 && j >= g.jb - 1 && j <= g.je + 1) {
        if (g.visc_breaking) {
            m9 = 1;
        } else {
            int p = 1;
            for (int b = -1; b <= 1; b++)
                for (int a = -1; a <= 1; a++) p *= new_mask(g, f, i + a, j + b);
            if (fabs_(ro(f.Eta + (id))) / tmax(ro(f.Depth + (id)), GC(min_depth_frc)) > GC(swe_eta_dep)) p = 0;
            m9 = (uint8_t)p;
        }
    }
    if (f.MASK9[id] != m9) *f.m9_dirty = 1;  // the tridiagonal matrices change
    f.MASK9[id] = m9;
}

template <typename T>
__global__ void __launch_bounds__(256) k_mask(Grid g, Fields<T> f) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i > g.Mloc || j > g.Nloc) return;
    mask_cell(g, f, i, j);
}

// ---------------------------------------------------------------------------
// BREAKING (breaker.F:87-353), default branch
// ---------------------------------------------------------------------------
template <typename T> struct BrkLocal {
    T tmp1, tmp2, tmp3, et;
};
template <typename T>
__device__ __forceinline__ BrkLocal<T> brk_local(const Grid &g, const Fields<T> &f, size_t id) {
    BrkLocal<T> b;
    b.tmp3 = fsqrt((T)GRAV * tmax(GC(min_depth_frc), ro(f.H + (id))));
    b.tmp1 = GC(cbrk1) * b.tmp3;
    b.tmp2 = GC(cbrk2) * b.tmp3;
    b.et = ro(f.ETAT + (id));
    return b;
}
template <typename T>
__device__ __forceinline__ bool in_wk_zone(const Grid &g, int i, int j) {
    const T xmk = i2r<T>(i - g.ib) * GC(DX), ymk = i2r<T>(j - g.jb) * GC(DY);
    return fabs_(xmk - GC(xc_wk)) < GC(width_wk) && fabs_(ymk - GC(yc_wk)) < GC(ywidth_wk) / (T)2;
}
template <typename T>
__device__ __forceinline__ T nu_value(const Grid &g, const Fields<T> &f, size_t id, const BrkLocal<T> &b, T age,
                                      bool zone) {
    const T mdf = GC(min_depth_frc);
    if (zone) {
        if (b.et > tmin(b.tmp2, GC(wavemaker_cbrk) * b.tmp3)) {
            const T cap1 = (T)1 * (tmax(ro(f.Depth + (id)), mdf) + ro(f.Eta + (id)));
            return cap1 * GC(wavemaker_cbrk) * b.tmp3 + GC(nu_bkg);
        }
        return (T)0 + GC(nu_bkg);
    }
    if (age > (T)0 && age < GC(T_brk) && b.et > b.tmp2) {
        const T cap1 = (T)1 * (tmax(ro(f.Depth + (id)), mdf) + ro(f.Eta + (id)));
        return cap1 * b.tmp2 + GC(nu_bkg);
    }
    return (T)0 + GC(nu_bkg);
}

// roller flux and undertow of a breaking cell (breaker.F:316-339):
// C1 = max(|ETAt|/tmp4, sqrt(g|H|)), R = min(|0.45 ETAt/max(C1,SMALL)|,
// 0.1638), ROLLER = |C1 - |u|| R (eta - ETAmean), UNDERTOW = -ROLLER times
// the direction cosines of ANGLE; 0.45 is a default-REAL literal and 0.1638
// a _SP one, so both enter FP64 as their float values.  ETAmean is zero
// until a mean is computed.
template <typename T>
__device__ __forceinline__ void roller_cell(const Grid &g, const Fields<T> &f, size_t id, T et) {
    const T ex = ro(f.ETAx + (id)), ey = ro(f.ETAy + (id));
    const T tmp4 = tmax(fsqrt(ex * ex + ey * ey), (T)SMALL);
    const T ANGLE = fatan2(-ey, -ex) * (T)180 / (T)PI_SP;
    const T C1 = tmax(fabs_(et) / tmp4, fsqrt((T)GRAV * fabs_(ro(f.H + (id)))));
    T R = fabs_((T)(double)0.45f * et / tmax(C1, (T)SMALL));
    R = tmin(R, (T)(double)0.1638f);
    const T u = f.U[id], v = f.V[id];
    const T em = g.stats ? f.ETAmean[id] : (T)0;
    const T rf = fabs_(C1 - fsqrt(u * u + v * v)) * R * (ro(f.Eta + (id)) - em);
    f.ROLLER[id] = rf;
    f.UNDERTOW_U[id] = -rf * fcos(ANGLE * (T)PI_SP / (T)180);
    f.UNDERTOW_V[id] = -rf * fsin(ANGLE * (T)PI_SP / (T)180);
}

// the breaking branch of the viscosity (outside the wavemaker zone)
template <typename T> __device__ __forceinline__ bool breaking_now(const Grid &g, const BrkLocal<T> &b, T age) {
    return age > (T)0 && age < GC(T_brk) && b.et > b.tmp2;
}

template <typename T>
__device__ __forceinline__ void break_cell(const Grid &g, const Fields<T> &f, int i, int j) {
    const size_t id = IDX(i, j);
    const T age = ro(f.AGE + (id));
    if (i < g.ib - 1 || i > g.ie + 1 || j < g.jb - 1 || j > g.je + 1) {
        f.AGEn[id] = age;
        return;
    }
    const T DT = DTV;
    const BrkLocal<T> b = brk_local(g, f, id);
    T an = age;
    bool cand = false;
    if (b.et >= b.tmp1 && (age == (T)0 || age > GC(T_brk))) an = DT;
    else if (age > (T)0) an = age + DT;
    else if (b.et >= b.tmp2) cand = true;
    f.AGEn[id] = an;
    const bool zone = in_wk_zone<T>(g, i, j);
    if (cand) {
        const int slot = atomicAdd(f.ncand, 1);
        f.cand[slot] = i + j * g.pitch;
    }
    if (zone || !cand) f.nu[id] = nu_value(g, f, id, b, an, zone);
    if (g.track_roller && !zone && !cand && breaking_now(g, b, an)) roller_cell(g, f, id, b.et);
}

template <typename T>
__global__ void __launch_bounds__(256) k_break_a(Grid g, Fields<T> f) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= g.Mloc || j >= g.Nloc) return;
    break_cell(g, f, i, j);
}

// The stage's GET_Eta_U_V_HU_HV tail, UPDATE_MASK and the parallel part of
// BREAKING in one pass: each reads only values that are final before it
// starts (U, V from the line solves; Eta, H from ESTIMATE_HUV; the MASK of
// the start of the stage; AGE of the previous stage) and writes disjoint
// arrays, so one thread can do all three.  Launched over (Mloc+1) x (Nloc+1).
template <typename T>
__global__ void __launch_bounds__(256) k_post_mask_break(Grid g, Fields<T> f) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i > g.Mloc || j > g.Nloc) return;
    if (i < g.Mloc && j < g.Nloc) {
        // the breaking and mask parts' inputs, read after the post part's stores
        const size_t id = IDX(i, j);
        prefetch_l1(f.ETAT + id);
        prefetch_l1(f.AGE + id);
        prefetch_l1(f.Eta + id);
        prefetch_l1(f.Depth + id);
        prefetch_l1(f.MASK_STRUC + id);
        // the post part's inputs, which it reads after a branch on MASK
        prefetch_l1(f.MASK + id);
        prefetch_l1(f.H + id);
        prefetch_l1(f.U + id);
        prefetch_l1(f.V + id);
        post_cell(g, f, i, j);
        break_cell(g, f, i, j);
    }
    mask_cell(g, f, i, j);
}

// the neighbour test of one candidate (breaker.F:182-224); N = new values
template <typename T>
__device__ __forceinline__ bool brk_neigh(const Grid &g, const Fields<T> &f, const volatile T *N, int i, int j,
                                          T DT) {
    const size_t id = IDX(i, j);
    const T ex = ro(f.ETAx + (id)), ey = ro(f.ETAy + (id));
    const T ANGLE = fatan2(-ey, -ex) * (T)180 / (T)PI_SP;
    const T tmp4 = tmax(fsqrt(ex * ex + ey * ey), (T)SMALL);
    const T Hc = ro(f.H + (id));
    const T C = tmin(fabs_(ro(f.ETAT + (id))) / tmp4, fsqrt((T)GRAV * fabs_(Hc)));
    const T DX = GC(DX), DY = GC(DY);
    const T propxy = fsqrt(DX * DX + DY * DY) / tmax(C, (T)SMALL);
    const T propx = fsqrt(DX * DX) / tmax(C, (T)SMALL);
    const T propy = fsqrt(DY * DY) / tmax(C, (T)SMALL);
    const T *O = f.AGE;  // values before the sweep
#define NW(a, b) N[IDX(i + (a), j + (b))]
#define OL(a, b) O[IDX(i + (a), j + (b))]
    bool hit = false;
    T A1, A2, A3;
    if (ANGLE >= (T)0 && ANGLE < (T)90) {
        A1 = NW(-1, 0);
        A2 = NW(-1, -1);
        A3 = NW(0, -1);
        if ((A1 >= DT && A1 > propx) || (A2 >= DT && A2 > propxy) || (A3 >= DT && A3 > propy)) hit = true;
    }
    if (ANGLE >= (T)90 && ANGLE < (T)180) {
        A1 = OL(1, 0);
        A2 = NW(1, -1);
        A3 = NW(0, -1);
        if ((A1 >= DT && A1 > propx) || (A2 >= DT && A2 > propxy) || (A3 >= DT && A3 > propy)) hit = true;
    }
    if (ANGLE >= (T)-180 && ANGLE < (T)-90) {
        A1 = OL(1, 0);
        A2 = OL(1, 1);
        A3 = OL(0, 1);
        if ((A1 >= DT && A1 > propx) || (A2 >= DT && A2 > propxy) || (A3 >= DT && A3 > propy)) hit = true;
    }
    if (ANGLE >= (T)-90 && ANGLE < (T)0) {
        A1 = OL(0, 1);
        A2 = OL(-1, 1);
        A3 = NW(-1, 0);
        if ((A1 >= DT && A1 > propy) || (A2 >= DT && A2 > propxy) || (A3 >= DT && A3 > propx)) hit = true;
    }
#undef NW
#undef OL
    return hit;
}

// one candidate of the sweep: 0 -> DT when a neighbour before it carries
// the age far enough (breaker.F:182-224)
template <typename T>
__device__ __forceinline__ bool brk_try(const Grid &g, const Fields<T> &f, volatile T *N, int code, T DT) {
    const int i = code % g.pitch, j = code / g.pitch;
    const size_t id = IDX(i, j);
    if (N[id] != (T)0 || !brk_neigh(g, f, N, i, j, DT)) return false;
    N[id] = DT;
    return true;
}

// exclusive prefix sum over a 1024-thread block (wsum: 32 ints of shared
// memory); returns this thread's prefix
__device__ __forceinline__ int block_scan_1024(int x, int *wsum) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int inc = x;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, inc, d);
        if (lane >= d) inc += y;
    }
    if (lane == 31) wsum[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        const int w = wsum[lane];
        int wi = w;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, wi, d);
            if (lane >= d) wi += y;
        }
        wsum[lane] = wi - w;
    }
    __syncthreads();
    const int r = wsum[warp] + inc - x;
    __syncthreads();
    return r;
}

// Candidates of the sweep, in one 1024-thread block, then nu.  The sweep
// (j outer, i inner) lets a candidate read the new values of (i-1,j),
// (i-1,j-1), (i,j-1), (i+1,j-1) (cells before it) and the old values of
// the cells after it, so new values only flow forward and a candidate
// turns from 0 to DT at most once.
//  - Passes to the fixed point: every candidate tests its neighbours in
//    parallel, and the pass repeats while any changed.  What a pass sets
//    is also set by the sequential sweep (by induction over the passes),
//    so the fixed point is its result.  A chain of k candidates that set
//    one another takes k + 1 passes; most stages need two or three.
//  - After g.brk_passes passes without the fixed point, the rest in one
//    pass by level t = i + 2j: the cells a candidate reads new values of
//    lie on levels t-1, t-3, t-2, t-1, the cells it reads old values of on
//    levels above t.  The candidates are sorted by level (a histogram, its
//    prefix sum and a scatter, into the line solver's tq and tp planes,
//    which are free between the stage's line solve and the next) and the
//    non-empty levels are worked in order, one barrier each.  Starting
//    from any pass's state (a subset of the sweep's result) this gives the
//    sweep's result, in time bounded by the candidates and the levels
//    (at most Mglob + 2 Nglob + 7) whatever the breaking pattern.
template <typename T>
__global__ void __launch_bounds__(1024) k_break_b(Grid g, Fields<T> f) {
    __shared__ int changed;
    __shared__ int wsum[32];
    __shared__ int lev_beg[1024], lev_end[1024];
    __shared__ unsigned nonempty[32];
    const int n = *f.ncand;
    const T DT = DTV;
    volatile T *N = f.AGEn;
    bool done = false;
    for (int pass = 0; pass < g.brk_passes && pass <= n; pass++) {
        if (threadIdx.x == 0) changed = 0;
        __syncthreads();
        for (int c = threadIdx.x; c < n; c += blockDim.x)
            if (brk_try(g, f, N, f.cand[c], DT)) changed = 1;
        __syncthreads();
        const int ch = changed;
        __syncthreads();
        if (!ch) {
            done = true;
            break;
        }
    }
    if (!done && n > 0) {
        // levels of the candidate range Ibeg-1..Iend+1 x Jbeg-1..Jend+1
        const int i0 = g.ib - 1, j0 = g.jb - 1;
        const int nlev = (g.ie + 1 - i0) + 2 * (g.je + 1 - j0) + 1;
        volatile int *off = reinterpret_cast<volatile int *>(f.tq);
        int *off_a = reinterpret_cast<int *>(f.tq);
        int *sorted = reinterpret_cast<int *>(f.tp);
        auto level = [&](int code) { return (code % g.pitch - i0) + 2 * (code / g.pitch - j0); };
        for (int t = threadIdx.x; t < nlev; t += 1024) off[t] = 0;
        __syncthreads();
        for (int c = threadIdx.x; c < n; c += 1024) atomicAdd(&off_a[level(f.cand[c])], 1);
        __syncthreads();
        // counts -> exclusive offsets: each thread takes a run of levels
        const int per = (nlev + 1023) / 1024;
        const int lo = min((int)threadIdx.x * per, nlev), hi = min(lo + per, nlev);
        int sum = 0;
        for (int t = lo; t < hi; t++) sum += off[t];
        int acc = block_scan_1024(sum, wsum);
        for (int t = lo; t < hi; t++) {
            const int v = off[t];
            off[t] = acc;
            acc += v;
        }
        __syncthreads();
        // scatter; afterwards off[t] is the end of level t
        for (int c = threadIdx.x; c < n; c += 1024) {
            const int code = f.cand[c];
            sorted[atomicAdd(&off_a[level(code)], 1)] = code;
        }
        __syncthreads();
        // the levels in order, 1024 at a time: each thread flags its level
        // if non-empty, and all threads walk the same flags, so every
        // thread reaches the same barriers
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        for (int t0 = 0; t0 < nlev; t0 += 1024) {
            const int t = t0 + threadIdx.x;
            int b = 0, e = 0;
            if (t < nlev) {
                e = off[t];
                b = t == 0 ? 0 : off[t - 1];
            }
            lev_beg[threadIdx.x] = b;
            lev_end[threadIdx.x] = e;
            const unsigned m = __ballot_sync(0xffffffffu, e > b);
            if (lane == 0) nonempty[warp] = m;
            __syncthreads();
            for (int w = 0; w < 32; w++) {
                unsigned mw = nonempty[w];
                while (mw) {
                    const int k = w * 32 + __ffs(mw) - 1;
                    mw &= mw - 1;
                    for (int c = lev_beg[k] + threadIdx.x; c < lev_end[k]; c += 1024)
                        brk_try(g, f, N, sorted[c], DT);
                    __syncthreads();
                }
            }
            __syncthreads();  // all have read the flags before the next chunk's
        }
    }
    for (int c = threadIdx.x; c < n; c += blockDim.x) {
        const int code = f.cand[c];
        const int i = code % g.pitch, j = code / g.pitch;
        const size_t id = IDX(i, j);
        if (in_wk_zone<T>(g, i, j)) continue;
        const BrkLocal<T> b = brk_local(g, f, id);
        f.nu[id] = nu_value(g, f, id, b, (T)N[id], false);
        if (g.track_roller && breaking_now(g, b, (T)N[id])) roller_cell(g, f, id, b.et);
    }
    __syncthreads();
    if (threadIdx.x == 0) *f.ncand = 0;
}

// ---------------------------------------------------------------------------
// EXCHANGE ghost fill (bc.F:426-529 with PHI_COLL / PHI_COLL_VARIABLE_LENGTH)
// in place.  One thread per ghost cell; in periodic mode the thread of an
// x-ghost cell also moves its pre-fill value into the corner cell that
// copies it (bc.F:735-740 runs before the x mirror).
// ---------------------------------------------------------------------------
struct GhostSet {
    int n;  // number of fields
};

template <typename T>
__device__ __forceinline__ void ghost_x_cell(const Grid &g, T *phi, int i, int j, int vtype) {
    // i is an x-ghost column, j an interior row
    const int si = mirror_x(g, i);
    const T v = phi[IDX(si, j)];
    if (g.periodic) {
        if (j >= g.je - 2) phi[IDX(i, j - (g.je - 2))] = phi[IDX(i, j)];
        if (j <= g.jb + 2) phi[IDX(i, j + g.je - 2)] = phi[IDX(i, j)];
    }
    phi[IDX(i, j)] = (vtype == 2) ? -v : v;
}
template <typename T>
__device__ __forceinline__ void ghost_y_cell(const Grid &g, T *phi, int i, int j, int vtype) {
    // j is a y-ghost row, any column
    const bool gx = (i < g.ib) || (i > g.ie);
    if (g.periodic) {
        if (gx) return;  // corner: written by the x-ghost thread
        phi[IDX(i, j)] = phi[IDX(i, period_y(g, j))];
        return;
    }
    const T v = phi[IDX(mirror_x(g, i), mirror_y(g, j))];
    T r = v;
    if (vtype == 2 && gx) r = -r;
    if (vtype == 3) r = -r;
    phi[IDX(i, j)] = r;
}

// EXCHANGE's PHI_COLL of Wsurf, P_center, Q_center, U_davg and V_davg
// (bc.F:438-443), scalar rules, after the last two stages
template <typename T>
__global__ void __launch_bounds__(256) k_ghost_rad(Grid g, Fields<T> f) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int nX = 6 * g.Nglob, nY = 6 * g.Mloc;
    if (t >= nX + nY) return;
    const size_t PL = (size_t)g.pitch * (size_t)(g.Nloc + 1);
    T *const planes[5] = {f.rad + RP_WS * PL, f.rad + RP_PC * PL, f.rad + RP_QC * PL, f.rad + RP_UD * PL,
                          f.rad + RP_VD * PL};
    if (t < nX) {
        const int col = t % 6;
        const int i = col < 3 ? col : g.ie + 1 + (col - 3);
        const int j = g.jb + t / 6;
#pragma unroll
        for (int k = 0; k < 5; k++) ghost_x_cell(g, planes[k], i, j, 1);
    } else {
        const int u = t - nX;
        const int row = u / g.Mloc;
        const int i = u % g.Mloc;
        const int j = row < 3 ? row : g.je + 1 + (row - 3);
#pragma unroll
        for (int k = 0; k < 5; k++) ghost_y_cell(g, planes[k], i, j, 1);
    }
}

template <typename T>
__global__ void __launch_bounds__(256) k_ghost(Grid g, Fields<T> f, int with_age) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int nX = 6 * g.Nglob;
    const int nY = 6 * g.Mloc;
    const int ncell = nX + nY;
    if (t < ncell) {
        if (t < nX) {
            const int col = t % 6;
            const int i = col < 3 ? col : g.ie + 1 + (col - 3);
            const int j = g.jb + t / 6;
            ghost_x_cell(g, f.Eta, i, j, 1);
            ghost_x_cell(g, f.U, i, j, 2);
            ghost_x_cell(g, f.HU, i, j, 2);
            ghost_x_cell(g, f.V, i, j, 3);
            ghost_x_cell(g, f.HV, i, j, 3);
            ghost_x_cell(g, f.MASK, i, j, 1);
            if (with_age) {
                ghost_x_cell(g, f.AGE, i, j, 1);
                ghost_x_cell(g, f.nu, i, j, 1);
            }
        } else {
            const int u = t - nX;
            const int row = u / g.Mloc;
            const int i = u % g.Mloc;
            const int j = row < 3 ? row : g.je + 1 + (row - 3);
            ghost_y_cell(g, f.Eta, i, j, 1);
            ghost_y_cell(g, f.U, i, j, 2);
            ghost_y_cell(g, f.HU, i, j, 2);
            ghost_y_cell(g, f.V, i, j, 3);
            ghost_y_cell(g, f.HV, i, j, 3);
            ghost_y_cell(g, f.MASK, i, j, 1);
            if (with_age) {
                ghost_y_cell(g, f.AGE, i, j, 1);
                ghost_y_cell(g, f.nu, i, j, 1);
            }
        }
        return;
    }
    if (!with_age) return;
    // P on x-faces and Q on y-faces: plain mirror on all four sides
    // (PHI_COLL_VARIABLE_LENGTH, periodic ignored), last index Iend1 / Jend1
    int u = t - ncell;
    const int nPX = 6 * g.Nglob, nPY = 6 * (g.Mloc + 1);
    if (u < nPX + nPY) {
        const int ie1 = g.ie + 1;
        int i, j;
        if (u < nPX) {
            const int col = u % 6;
            i = col < 3 ? col : ie1 + 1 + (col - 3);
            j = g.jb + u / 6;
        } else {
            u -= nPX;
            const int row = u / (g.Mloc + 1);
            i = u % (g.Mloc + 1);
            j = row < 3 ? row : g.je + 1 + (row - 3);
        }
        const int si = i < g.ib ? 2 * g.ib - 1 - i : (i > ie1 ? 2 * ie1 + 1 - i : i);
        const int sj = mirror_y(g, j);
        f.P[IDX(i, j)] = f.P[IDX(si, sj)];
        return;
    }
    u -= nPX + nPY;
    const int nQX = 6 * (g.Nglob + 1), nQY = 6 * g.Mloc;
    if (u < nQX + nQY) {
        const int je1 = g.je + 1;
        int i, j;
        if (u < nQX) {
            const int col = u % 6;
            i = col < 3 ? col : g.ie + 1 + (col - 3);
            j = g.jb + u / 6;
        } else {
            u -= nQX;
            const int row = u / g.Mloc;
            i = u % g.Mloc;
            j = row < 3 ? row : je1 + 1 + (row - 3);
        }
        const int si = mirror_x(g, i);
        const int sj = j < g.jb ? 2 * g.jb - 1 - j : (j > je1 ? 2 * je1 + 1 - j : j);
        f.Q[IDX(i, j)] = f.Q[IDX(si, sj)];
    }
}

// U,V,HU,HV *= MASK (bc.F:491-494) and, optionally, SPONGE_DAMPING
// (sponge.F:52-66), on every cell
template <typename T>
__global__ void __launch_bounds__(256) k_maskmul(Grid g, Fields<T> f, int sponge) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= g.Mloc || j >= g.Nloc) return;
    const size_t id = IDX(i, j);
    // every load before the first store (see k_begin)
    const uint8_t mi = f.MASK[id];
    const T m = m2r<T>(mi);
    const T u0 = f.U[id], v0 = f.V[id], hu = f.HU[id], hv = f.HV[id];
    const T s = sponge ? f.SPONGE[id] : (T)1;
    const T eta = (sponge && mi > 0) ? f.Eta[id] : (T)0;
    T u = u0 * m, v = v0 * m;
    f.HU[id] = hu * m;
    f.HV[id] = hv * m;
    if (sponge) {
        if (mi > 0) f.Eta[id] = eta / s;
        u = u / s;
        v = v / s;
    }
    f.U[id] = u;
    f.V[id] = v;
}

// SPONGE_DAMPING alone
template <typename T>
__global__ void k_sponge(Grid g, Fields<T> f) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= g.Mloc || j >= g.Nloc) return;
    const size_t id = IDX(i, j);
    const T s = f.SPONGE[id];
    if (f.MASK[id] > 0) f.Eta[id] = f.Eta[id] / s;
    f.U[id] = f.U[id] / s;
    f.V[id] = f.V[id] / s;
}

// ---------------------------------------------------------------------------
// ESTIMATE_DT (misc.F:216-296): CFL minimum over every cell, then DT and
// TIME on the device.  Positive doubles order like their bit patterns.
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ T dt_val(const Grid &g, T H, T U, T V) {
    const T c = fsqrt((T)GRAV * tmax(H, GC(min_depth_frc)));
    T t1 = fabs_(U) + c;
    T t2 = (t1 < (T)SMALL) ? GC(DX) / (T)SMALL : GC(DX) / t1;
    T m = t2;
    t1 = fabs_(V) + c;
    t2 = (t1 < (T)SMALL) ? GC(DY) / (T)SMALL : GC(DY) / t1;
    if (t2 < m) m = t2;
    return m;
}
template <typename T>
__device__ __forceinline__ T dt_cell(const Grid &g, const Fields<T> &f, size_t id) {
    return dt_val(g, f.H[id], f.U[id], f.V[id]);
}

__device__ __forceinline__ double tminr(double a, double b) { return fmin(a, b); }
__device__ __forceinline__ float tminr(float a, float b) { return fminf(a, b); }

// block minimum in T, then one atomicMin on the (order-preserving) bits of
// the positive double
template <typename T>
__device__ __forceinline__ void block_min_to_global(T v, unsigned long long *dst) {
    __shared__ T sm[32];
    for (int o = 16; o > 0; o >>= 1) v = tminr(v, __shfl_xor_sync(0xffffffffu, v, o));
    const int lane = (threadIdx.x + threadIdx.y * blockDim.x) & 31;
    const int warp = (threadIdx.x + threadIdx.y * blockDim.x) >> 5;
    const int nw = (blockDim.x * blockDim.y + 31) >> 5;
    if (lane == 0) sm[warp] = v;
    __syncthreads();
    if (warp == 0) {
        v = lane < nw ? sm[lane] : (T)1.0e30;
        for (int o = 16; o > 0; o >>= 1) v = tminr(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (lane == 0) atomicMin(dst, (unsigned long long)__double_as_longlong((double)v));
    }
}

// Eta0 = Eta on the ghost ring, before the step's EXCHANGE refills it
// (main.F:295 comes before main.F:313): the ring still holds the previous
// step's sponge-damped values.  6*Mloc + 6*Nglob cells, one thread each.
template <typename T>
__global__ void __launch_bounds__(256) k_eta0_ring(Grid g, Fields<T> f) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    int i, j;
    if (t < 3 * g.Mloc) {
        j = t / g.Mloc;
        i = t - j * g.Mloc;
    } else if ((t -= 3 * g.Mloc) < 3 * g.Mloc) {
        j = g.Nloc - 3 + t / g.Mloc;
        i = t % g.Mloc;
    } else if ((t -= 3 * g.Mloc) < 6 * g.Nglob) {
        j = NG + t / 6;
        const int c = t % 6;
        i = c < 3 ? c : g.Mloc - 6 + c;
    } else {
        return;
    }
    f.Eta0[IDX(i, j)] = f.Eta[IDX(i, j)];
}

// begin of a step: U,V,HU,HV *= MASK after the ghost fill, the Eta0
// (interior; the ring is copied by k_eta0_ring before the fill), Ubar0,
// Vbar0, U0, V0 copies (main.F:295-297,331) and the CFL minimum
template <typename T>
__global__ void __launch_bounds__(256) k_begin(Grid g, Fields<T> f) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    T v = (T)1.0e30;
    if (i < g.Mloc && j < g.Nloc) {
        const size_t id = IDX(i, j);
        // every load before the first store: the copies' sources and
        // destinations are different arrays, which the compiler cannot know
        const bool in = i >= g.ib && i <= g.ie && j >= g.jb && j <= g.je;
        const T m = m2r<T>(f.MASK[id]);
        const T u0 = f.U[id], v0 = f.V[id], hu = f.HU[id], hv = f.HV[id];
        const T ub = f.Ubar[id], vb = f.Vbar[id], h = f.H[id];
        const T eta = in ? f.Eta[id] : (T)0;
        const T u = u0 * m, vv = v0 * m;
        f.U[id] = u;
        f.V[id] = vv;
        f.HU[id] = hu * m;
        f.HV[id] = hv * m;
        if (in) f.Eta0[id] = eta;
        f.Ubar0[id] = ub;
        f.Vbar0[id] = vb;
        f.U0[id] = u;
        f.V0[id] = vv;
        v = dt_val(g, h, u, vv);
    }
    block_min_to_global(v, f.dtmin_bits);
}

template <typename T>
__global__ void __launch_bounds__(256) k_dt_only(Grid g, Fields<T> f) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    T v = (T)1.0e30;
    if (i < g.Mloc && j < g.Nloc) v = dt_cell(g, f, IDX(i, j));
    block_min_to_global(v, f.dtmin_bits);
}

// DT = CFL*min (with DT_fixed halving), TIME += DT, and the JON_2D
// cos/sin(omega_k TIME) table of this step (sources.F:121-124)
static __global__ void k_dt_final(Grid g, double *dsc, float *fsc, unsigned long long *bits, double *omega,
                                  double *wmcs, float *wmcsf, int nfreq) {
    __shared__ double time_s;
    if (threadIdx.x == 0) {
        double tmp3 = __longlong_as_double((long long)*bits);
        if (!(tmp3 < LARGE)) tmp3 = LARGE;
        const double dt_tmp = g.cfl * tmp3;
        double dt;
        if (g.fixed_dt) {
            dt = g.dt_fixed;
            for (int k = 0; k < 4096 && dt > dt_tmp; k++) dt = dt / 2.0;
        } else {
            dt = dt_tmp;
        }
        dsc[S_DT] = dt;
        dsc[S_TIME] = dsc[S_TIME] + dt;
        time_s = dsc[S_TIME];
        *bits = 0x7ff0000000000000ull;  // +inf for the next minimum
        // float scalars of the step for the mixed path: DT, 1/DT, the
        // wavemaker ramp (sources.F:110,120) and the WK_REG phase
        // 2*pi/Tperiod*TIME reduced modulo 2*pi
        fsc[FS_DT] = (float)dt;
        fsc[FS_RDT] = (float)(1.0 / dt);
        if (g.wavemaker == FW_WK_REG) {
            fsc[FS_WKAA] = (float)(tanh(PI_SP / (g.time_ramp * g.tperiod) * time_s) * g.D_gen);
            const double ph = 2.0 * PI_SP / g.tperiod * time_s;
            fsc[FS_WKPH] = (float)(ph - 2.0 * PI_SP * floor(ph / (2.0 * PI_SP)));
        } else if (g.wavemaker == FW_WK_JON_2D) {
            fsc[FS_WKAA] = (float)tanh(PI_SP / (g.time_ramp / g.freq_peak) * time_s);
        }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < nfreq; k += blockDim.x) {
        wmcs[2 * k] = cos(omega[k] * time_s);
        wmcs[2 * k + 1] = sin(omega[k] * time_s);
        wmcsf[2 * k] = (float)wmcs[2 * k];
        wmcsf[2 * k + 1] = (float)wmcs[2 * k + 1];
    }
}

// ---------------------------------------------------------------------------
// end of a step: MAX_MIN_PROPERTY (Hmax, misc.F:307-383) and the
// CHECK_BLOWUP maximum (misc.F:394-433)
// ---------------------------------------------------------------------------
// MIXING_STUFF's T_sum (mixing.F:60, 143-144, 224): one thread, before
// k_end; S_MFLAG tells k_end what to do with the cells this step
static __global__ void k_tsum(Grid g, double *dsc, float *fsc) {
    int flag = 0;
    double ts = dsc[S_TSUM], tsu = ts;
    if (dsc[S_TIME] >= g.steady_time) {
        ts = ts + dsc[S_DT];
        tsu = ts;
        if (ts >= g.t_intv_mean) {
            flag = 2;
            ts = ts - g.t_intv_mean;
            dsc[S_NMEAN] = dsc[S_NMEAN] + 1.0;
        } else {
            flag = 1;
        }
    }
    dsc[S_TSUM] = ts;
    dsc[S_TSUMU] = tsu;
    dsc[S_MFLAG] = (double)flag;
    fsc[FS_TSUM] = (float)tsu;
}

// s += x with Kahan compensation k (mixed path), s = x + s otherwise
template <typename T> __device__ __forceinline__ void stat_add(T *s, T *k, size_t id, T x) {
    if constexpr (sizeof(T) == sizeof(double)) {
        s[id] = x + s[id];
    } else {
        const float y = __fsub_rn(x, k[id]);
        const float t = __fadd_rn(s[id], y);
        k[id] = __fsub_rn(__fsub_rn(t, s[id]), y);
        s[id] = t;
    }
}
// the compensated value of a sum
template <typename T> __device__ __forceinline__ T stat_val(const T *s, const T *k, size_t id) {
    if constexpr (sizeof(T) == sizeof(double)) return s[id];
    else return __fsub_rn(s[id], k[id]);
}

// CALCULATE_MEAN's radiation-stress, momentum-flux and breaking-dissipation
// sums at one cell (mixing.F:156-167, 270-281), with the ETAmean the
// caller's branch has at that point and the last interval's U_davg_mean
template <typename T> __device__ __forceinline__ void rad_sums(const Grid &g, const Fields<T> &f, size_t id, T DT,
                                                               T etamean) {
    const size_t PL = (size_t)g.pitch * (size_t)(g.Nloc + 1);
    T *const r = f.rad;
    T *const ks = sizeof(T) == sizeof(float) ? r + RP_KAHAN * PL : nullptr;
#define RV(k) r[(size_t)(k) * PL + id]
#define SUM(k, x) stat_add(r + (RP_SUM + (k)) * PL, ks ? ks + (size_t)(k) * PL : nullptr, id, (T)(x))
    const T udv = RV(RP_UD), vdv = RV(RP_VD);
    const T ud = udv - RV(RP_MEAN + 0), vd = vdv - RV(RP_MEAN + 1);
    const T hd = f.Eta[id] - etamean + f.Depth[id];
    const T u = f.U[id], v = f.V[id], w = RV(RP_WS);
    const T sp = fsqrt(u * u + v * v);
    SUM(0, udv * DT);
    SUM(1, vdv * DT);
    SUM(2, RV(RP_PC) * DT);
    SUM(3, RV(RP_QC) * DT);
    SUM(4, ud * ud * hd * DT);
    SUM(5, ud * vd * hd * DT);
    SUM(6, vd * vd * hd * DT);
    SUM(7, (T)0.25 * w * w * hd * DT);
    SUM(8, u * sp * DT);
    SUM(9, v * sp * DT);
    SUM(10, RV(RP_BX) * DT);
    SUM(11, RV(RP_BY) * DT);
#undef SUM
#undef RV
}
// the means at the end of an interval, then the sums restart
template <typename T> __device__ __forceinline__ void rad_means(const Grid &g, const Fields<T> &f, size_t id, T Ts) {
    const size_t PL = (size_t)g.pitch * (size_t)(g.Nloc + 1);
    T *const r = f.rad;
#pragma unroll
    for (int k = 0; k < 12; k++) {
        T *s = r + (RP_SUM + k) * PL;
        T *kk = sizeof(T) == sizeof(float) ? r + (RP_KAHAN + k) * PL : nullptr;
        r[(RP_MEAN + k) * PL + id] = stat_val(s, kk, id) / Ts;
        s[id] = (T)0;
        if (kk) kk[id] = (T)0;
    }
}

// CALCULATE_MEAN (mixing.F:141-301) at one cell: the Eta, U, V and
// (Eta-ETAmean)^2 time sums, their means at the end of an interval, and the
// zero-up-crossing wave heights; the float path keeps the sums compensated
template <typename T> __device__ __forceinline__ void mean_cell(const Grid &g, const Fields<T> &f, size_t id,
                                                                int flag) {
    const T DT = DTV;
    const T eta = f.Eta[id], u = f.U[id], v = f.V[id];
    const T d = eta - f.ETAmean[id];
    if (flag == 2) {
        T Ts;
        if constexpr (sizeof(T) == sizeof(double)) Ts = f.dsc[S_TSUMU];
        else Ts = f.fsc[FS_TSUM];
        stat_add(f.ETA2sum, f.kETA2sum, id, d * d * DT);
        const T e2 = stat_val(f.ETA2sum, f.kETA2sum, id) / Ts;
        f.ETA2mean[id] = e2;
        stat_add(f.Usum, f.kUsum, id, u * DT);
        stat_add(f.Vsum, f.kVsum, id, v * DT);
        stat_add(f.ETAsum, f.kETAsum, id, eta * DT);
        f.Umean[id] = stat_val(f.Usum, f.kUsum, id) / Ts;
        f.Vmean[id] = stat_val(f.Vsum, f.kVsum, id) / Ts;
        const T em = stat_val(f.ETAsum, f.kETAsum, id) / Ts;
        f.ETAmean[id] = em;
        if (f.rad) {
            rad_sums(g, f, id, DT, em);
            rad_means(g, f, id, Ts);
        }
        f.Usum[id] = (T)0;
        f.Vsum[id] = (T)0;
        f.ETAsum[id] = (T)0;
        f.ETA2sum[id] = (T)0;
        if constexpr (sizeof(T) == sizeof(float)) {
            f.kUsum[id] = 0.0f;
            f.kVsum[id] = 0.0f;
            f.kETAsum[id] = 0.0f;
            f.kETA2sum[id] = 0.0f;
        }
        f.SigWH[id] = (T)C4004_SP * fsqrt(e2);
        const T nz = f.NZU[id];
        if (nz >= (T)2) {
            f.WHave[id] = f.HavgSum[id] / nz;
            f.WHrms[id] = fsqrt(f.HrmsSum[id] / nz);
        }
    } else {
        stat_add(f.Usum, f.kUsum, id, u * DT);
        stat_add(f.Vsum, f.kVsum, id, v * DT);
        stat_add(f.ETAsum, f.kETAsum, id, eta * DT);
        stat_add(f.ETA2sum, f.kETA2sum, id, d * d * DT);
        if (f.rad) rad_sums(g, f, id, DT, f.ETAmean[id]);
        T emax = f.Emax[id], emin = f.Emin[id];
        if (eta > emax) emax = eta;
        if (eta < emin) emin = eta;
        const T tmp0 = f.Eta0[id] - f.ETAmean[id];
        if (d > tmp0 && d * tmp0 <= (T)0) {
            const T nz = f.NZU[id] + (T)1;
            f.NZU[id] = nz;
            if (nz >= (T)2) {
                const T h = emax - emin;
                f.HavgSum[id] = (f.HavgSum[id] + emax) - emin;  // left to right (mixing.F:293)
                f.HrmsSum[id] = f.HrmsSum[id] + h * h;
            }
            emax = (T)-1000;
            emin = (T)1000;
        }
        f.Emax[id] = emax;
        f.Emin[id] = emin;
    }
}

// the end of a CALCULATE_MEAN interval (mixing.F:183-219): the gradient
// fields DxSxx .. DxUVH of the new means on the interior, and FRCXmean,
// FRCYmean times Cd there.  Runs after k_end; a no-op on other steps.  The
// literals 9.80 and 0.5*9.80 are default REAL.
template <typename T>
__global__ void __launch_bounds__(256) k_rad_derived(Grid g, Fields<T> f) {
    if ((int)f.dsc[S_MFLAG] != 2) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x + g.ib;
    const int j = blockIdx.y * blockDim.y + threadIdx.y + g.jb;
    if (i > g.ie || j > g.je) return;
    const size_t PL = (size_t)g.pitch * (size_t)(g.Nloc + 1);
    const size_t id = IDX(i, j), e = IDX(i + 1, j), w = IDX(i - 1, j), n = IDX(i, j + 1), s = IDX(i, j - 1);
    T *const r = f.rad;
    const T *M = r + RP_MEAN * PL;
#define MN(k, c) M[(size_t)(k) * PL + (c)]
    const T DX = GC(DX), DY = GC(DY), mdf = GC(min_depth_frc);
    const T g98 = (T)9.80f, g49 = (T)(0.5f * 9.80f);
    const T *E2 = f.ETA2mean, *EM = f.ETAmean, *D = f.Depth;
    T *O = r + RP_DER * PL;
    // UU 4, UV 5, VV 6, WW 7; P 2, Q 3
    O[0 * PL + id] = (MN(4, e) - MN(4, w)) / (T)2 / DX - (MN(7, e) - MN(7, w)) / (T)2 / DX +
                     g49 * (E2[e] - E2[w]) / (T)2 / DX;
    O[1 * PL + id] = (MN(5, n) - MN(5, s)) / (T)2 / DY;
    O[2 * PL + id] = (MN(6, n) - MN(6, s)) / (T)2 / DY - (MN(7, n) - MN(7, s)) / (T)2 / DY +
                     g49 * (E2[n] - E2[s]) / (T)2 / DY;
    O[3 * PL + id] = (MN(5, e) - MN(5, w)) / (T)2 / DX;
    O[4 * PL + id] = g98 * (D[id] + EM[id]) * (EM[e] - EM[w]) / (T)2 / DX;
    O[5 * PL + id] = g98 * (D[id] + EM[id]) * (EM[n] - EM[s]) / (T)2 / DY;
    const T he = tmax(D[e] + EM[e], mdf), hw = tmax(D[w] + EM[w], mdf);
    const T hn = tmax(D[n] + EM[n], mdf), hs = tmax(D[s] + EM[s], mdf);
    O[6 * PL + id] = (MN(2, e) * MN(2, e) / he - MN(2, w) * MN(2, w) / hw) / (T)2 / DX;
    O[7 * PL + id] = (MN(2, n) * MN(3, n) / hn - MN(2, s) * MN(3, s) / hs) / (T)2 / DY;
    O[8 * PL + id] = (MN(3, n) * MN(3, n) / hn - MN(3, s) * MN(3, s) / hs) / (T)2 / DY;
    O[9 * PL + id] = (MN(2, e) * MN(3, e) / he - MN(2, w) * MN(3, w) / hw) / (T)2 / DX;
    T *FX = r + (RP_MEAN + 8) * PL, *FY = r + (RP_MEAN + 9) * PL;
    FX[id] = FX[id] * f.Cd[id];
    FY[id] = FY[id] * f.Cd[id];
#undef MN
}

template <typename T>
__global__ void __launch_bounds__(256) k_end(Grid g, Fields<T> f, int track_hmax) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    T v = (T)0;
    const int mflag = g.stats ? (int)f.dsc[S_MFLAG] : 0;
    if (i < g.Mloc && j < g.Nloc) {
        const size_t id = IDX(i, j);
        if (mflag) mean_cell(g, f, id, mflag);
        const T eta = f.Eta[id];
        // MAX_MIN_PROPERTY (misc.F:323-350), wet cells
        if (f.MASK[id] > 0) {
            if (track_hmax && eta > f.Hmax[id]) f.Hmax[id] = eta;
            if (g.track_hmin && eta < f.Hmin[id]) f.Hmin[id] = eta;
            if (g.track_umax || g.track_mfmax) {
                const T u = f.U[id], w = f.V[id];
                if (g.track_umax) {
                    const T mv = fsqrt(u * u + w * w);
                    if (mv > f.Umax[id]) f.Umax[id] = mv;
                }
                if (g.track_mfmax) {
                    const T mv = (u * u + w * w) * (f.H[id]);
                    if (mv > f.MFmax[id]) f.MFmax[id] = mv;
                }
            }
        }
        if (i >= g.ib && i <= g.ie && j >= g.jb && j <= g.je) {
            const T a = fabs_(eta);
            v = (a == a) ? a : (T)INFINITY;  // NaN -> +inf
        }
    }
    // block maximum, then one atomicMax per block on the (order-preserving)
    // bits of the non-negative double
    __shared__ T sm[32];
    for (int o = 16; o > 0; o >>= 1) {
        const T w = __shfl_xor_sync(0xffffffffu, v, o);
        v = w > v ? w : v;
    }
    const int t = threadIdx.x + threadIdx.y * blockDim.x;
    const int nw = (blockDim.x * blockDim.y + 31) >> 5;
    if ((t & 31) == 0) sm[t >> 5] = v;
    __syncthreads();
    if (t < 32) {
        v = t < nw ? sm[t] : (T)0;
        for (int o = 16; o > 0; o >>= 1) {
            const T w = __shfl_xor_sync(0xffffffffu, v, o);
            v = w > v ? w : v;
        }
        if (t == 0) atomicMax(f.etamax_bits, (unsigned long long)__double_as_longlong((double)v));
    }
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
static inline dim3 grid2(int nx, int ny, dim3 b) { return dim3((nx + b.x - 1) / b.x, (ny + b.y - 1) / b.y); }
static const dim3 B2D(32, 8);
// blocks of k_flux: tiles of FX x FY faces over (Mglob+1) x Nglob x-faces
// or Mglob x (Nglob+1) y-faces
template <typename T, int DIR, int FY_ = flux_fy_default<T, DIR>()> static dim3 flux_grid(const Grid &g) {
    using TL = FluxTile<T, DIR, FY_>;
    const int w = DIR == 0 ? g.Mglob + 1 : g.Mglob, h = DIR == 0 ? g.Nglob : g.Nglob + 1;
    return dim3((w + TL::FX - 1) / TL::FX, (h + TL::FY - 1) / TL::FY);
}

static inline void note(fw_ctx *c, int n = 1) {
    c->launches += n;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess && !c->sticky_error) c->sticky_error = (int)e;
}

template <typename T> void launch_ghost(fw_ctx *c, bool full) {
    const Grid &g = c->g;
    int n = 6 * g.Nglob + 6 * g.Mloc;
    if (full) n += 6 * g.Nglob + 6 * (g.Mloc + 1) + 6 * (g.Nglob + 1) + 6 * g.Mloc;
    k_ghost<T><<<(n + 255) / 256, 256, 0, c->stream>>>(g, c->F<T>(), full ? 1 : 0);
    note(c);
}

template <typename T> void launch_exchange(fw_ctx *c, bool with_sponge) {
    const Grid &g = c->g;
    launch_ghost<T>(c, g.visc_breaking != 0);
    k_maskmul<T><<<grid2(g.Mloc, g.Nloc, c->blk(TK_MASKMUL)), c->blk(TK_MASKMUL), 0, c->stream>>>(g, c->F<T>(), with_sponge ? 1 : 0);
    note(c);
}

template <typename T> void launch_sponge(fw_ctx *c) {
    const Grid &g = c->g;
    k_sponge<T><<<grid2(g.Mloc, g.Nloc, B2D), B2D, 0, c->stream>>>(g, c->F<T>());
    note(c);
}

static void launch_dt_final(fw_ctx *c) {
    const bool d = c->p.precision == FW_PREC_FP64;
    double *dsc = d ? c->fd.dsc : c->ff.dsc;
    float *fsc = d ? c->fd.fsc : c->ff.fsc;
    unsigned long long *bits = d ? c->fd.dtmin_bits : c->ff.dtmin_bits;
    double *om = d ? c->fd.omega : c->ff.omega;
    double *cs = d ? c->fd.wmcs : c->ff.wmcs;
    float *csf = d ? c->fd.wmcsf : c->ff.wmcsf;
    k_dt_final<<<1, 128, 0, c->stream>>>(c->g, dsc, fsc, bits, om, cs, csf,
                                         c->g.wavemaker == FW_WK_JON_2D ? c->g.nfreq : 0);
    note(c);
}

template <typename T> void launch_estimate_dt(fw_ctx *c) {
    const Grid &g = c->g;
    k_dt_only<T><<<grid2(g.Mloc, g.Nloc, B2D), B2D, 0, c->stream>>>(g, c->F<T>());
    note(c);
    launch_dt_final(c);
}

template <typename T> void launch_begin_step(fw_ctx *c) {
    const Grid &g = c->g;
    const int nring = 6 * g.Mloc + 6 * g.Nglob;
    k_eta0_ring<T><<<(nring + 255) / 256, 256, 0, c->stream>>>(g, c->F<T>());
    note(c);
    launch_ghost<T>(c, g.visc_breaking != 0);
    k_begin<T><<<grid2(g.Mloc, g.Nloc, B2D), B2D, 0, c->stream>>>(g, c->F<T>());
    note(c);
    launch_dt_final(c);
}

template <typename T> void launch_dispersion(fw_ctx *c) {
    const Grid &g = c->g;
    k_disp_a<T><<<grid2(g.Mloc, g.Nloc, c->blk(TK_DISP_A)), c->blk(TK_DISP_A), 0, c->stream>>>(g, c->F<T>());
    note(c);
    k_disp_b<T><<<grid2(g.Mloc, g.Nloc, c->blk(TK_DISP_B)), c->blk(TK_DISP_B), 0, c->stream>>>(g, c->F<T>());
    note(c);
}

// the compiled flux tile heights: 8, 16 or 32 faces in float; 8 or 16 in
// double (a 32-high tile of doubles would not fit 48 KB)

template <typename T, int DIR, int FY_> static void flux_at(fw_ctx *c) {
    k_flux<T, DIR, FY_><<<flux_grid<T, DIR, FY_>(c->g), B2D, 0, c->stream>>>(c->g, c->F<T>());
}

// the TMA-staged flux kernel with the maps of the current MASK buffer (its
// shared-memory size is set when the maps are made, outside any capture)
template <typename T, int DIR, int FY_> static void flux_tma_at(fw_ctx *c) {
    using S = FluxStage<T, DIR, FY_>;
    const int fi = FY_ == 8 ? 0 : (FY_ == 16 ? 1 : 2);
    const int mi = ((const void *)c->F<T>().MASK == c->fmask_base[0]) ? 0 : 1;
    k_flux_tma<T, DIR, FY_><<<flux_grid<T, DIR, FY_>(c->g), B2D, S::BYTES, c->stream>>>(c->g, c->F<T>(),
                                                                                        c->fmaps[DIR][fi][mi]);
}
template <typename T, int DIR, int FY_> bool flux_tma_attr() {
    return cudaFuncSetAttribute(k_flux_tma<T, DIR, FY_>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                FluxStage<T, DIR, FY_>::BYTES) == cudaSuccess;
}
template <typename T> bool flux_tma_attrs() {
    bool ok = flux_tma_attr<T, 0, 8>() && flux_tma_attr<T, 0, 16>() && flux_tma_attr<T, 1, 8>() &&
              flux_tma_attr<T, 1, 16>();
    if constexpr (sizeof(T) == sizeof(float)) ok = ok && flux_tma_attr<T, 0, 32>() && flux_tma_attr<T, 1, 32>();
    return ok;
}

template <typename T, int DIR> static void launch_flux(fw_ctx *c) {
    const int fy = c->tune[TUNE_FLUX + DIR];
    if (c->tune[TUNE_FLUX_TMA + DIR] && c->fmaps_ok) {
        if (fy == 8) flux_tma_at<T, DIR, 8>(c);
        else if (fy == 16 || sizeof(T) == sizeof(double)) flux_tma_at<T, DIR, 16>(c);
        else if constexpr (sizeof(T) == sizeof(float)) flux_tma_at<T, DIR, 32>(c);
        note(c);
        return;
    }
    if constexpr (sizeof(T) == sizeof(float)) {
        if (fy == 8) flux_at<T, DIR, 8>(c);
        else if (fy == 16) flux_at<T, DIR, 16>(c);
        else flux_at<T, DIR, 32>(c);
    } else {
        if (fy == 8) flux_at<T, DIR, 8>(c);
        else flux_at<T, DIR, 16>(c);
    }
    note(c);
}

template <typename T> void launch_fluxes(fw_ctx *c) {
    launch_flux<T, 0>(c);
    launch_flux<T, 1>(c);
}

template <typename T> void launch_sources_debug(fw_ctx *c) {
    const Grid &g = c->g;
    k_sources<T><<<grid2(g.Mglob, g.Nglob, B2D), B2D, 0, c->stream>>>(g, c->F<T>());
    note(c);
}

template <typename T, int DIR, bool PER>
static bool launch_tri(fw_ctx *c, const LinePart &lp, bool fac = true, bool clear_dirty = false) {
    const Grid &g = c->g;
    const int nt = lp.nlines * lp.P;
    if constexpr (sizeof(T) == sizeof(float)) if (c->factored) {
        if (fac) {
            k_fac_a<T, DIR, PER><<<(nt + 127) / 128, 128, 0, c->stream>>>(g, c->F<T>(), lp);
            k_fac_b<T, DIR, PER><<<(lp.nlines + 127) / 128, 128, 0, c->stream>>>(g, c->F<T>(), lp);
            note(c, 2);
        }
        const size_t smem = lsx_smem_floats(lp.L, lp.P) * sizeof(float);
        if (DIR == 0 && !PER && lp.P <= 256 && smem <= 200 * 1024) {
            // lines of up to 2048 cells keep their per-cell coefficients in registers
            auto kern = lp.L <= 2048 ? k_linesolve_x<T, 8> : k_linesolve_x<T, 0>;
            if (smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            kern<<<lp.nlines, 256, smem, c->stream>>>(g, c->F<T>(), lp, clear_dirty ? 1 : 0);
            note(c);
            return clear_dirty;
        }
        const dim3 gi = grid2(g.Mglob, g.Nglob, B2D);
        const int nb = std::min(512, ((2 * lp.P + 31) / 32) * 32);
        const size_t sb = (size_t)16 * lp.P * sizeof(float);
        const unsigned ga = (unsigned)((nt + 127) / 128);
        // chunks of 16 rows (lines of 512 cells and more) walk in registers
        if (lp.m == 16) {
            k_sol_a<T, DIR, PER, 0, 16><<<ga, 128, 0, c->stream>>>(g, c->F<T>(), lp);
            k_sol_b<T, DIR, PER, 0><<<lp.nlines, nb, sb, c->stream>>>(g, c->F<T>(), lp);
            k_sol_c<T, DIR, 0, 16><<<ga, 128, 0, c->stream>>>(g, c->F<T>(), lp);
            k_resid<T, DIR, PER><<<gi, B2D, 0, c->stream>>>(g, c->F<T>(), lp);
            k_sol_a<T, DIR, PER, 1, 16><<<ga, 128, 0, c->stream>>>(g, c->F<T>(), lp);
            k_sol_b<T, DIR, PER, 1><<<lp.nlines, nb, sb, c->stream>>>(g, c->F<T>(), lp);
            k_sol_c<T, DIR, 1, 16><<<ga, 128, 0, c->stream>>>(g, c->F<T>(), lp);
        } else {
            k_sol_a<T, DIR, PER, 0, 0><<<ga, 128, 0, c->stream>>>(g, c->F<T>(), lp);
            k_sol_b<T, DIR, PER, 0><<<lp.nlines, nb, sb, c->stream>>>(g, c->F<T>(), lp);
            k_sol_c<T, DIR, 0, 0><<<ga, 128, 0, c->stream>>>(g, c->F<T>(), lp);
            k_resid<T, DIR, PER><<<gi, B2D, 0, c->stream>>>(g, c->F<T>(), lp);
            k_sol_a<T, DIR, PER, 1, 0><<<ga, 128, 0, c->stream>>>(g, c->F<T>(), lp);
            k_sol_b<T, DIR, PER, 1><<<lp.nlines, nb, sb, c->stream>>>(g, c->F<T>(), lp);
            k_sol_c<T, DIR, 1, 0><<<ga, 128, 0, c->stream>>>(g, c->F<T>(), lp);
        }
        note(c, 7);
        return false;
    }
    if constexpr (sizeof(T) == sizeof(double)) {
        k_thomas_rows<T, DIR, PER><<<grid2(g.Mglob, g.Nglob, B2D), B2D, 0, c->stream>>>(g, c->F<T>(), lp);
        k_thomas_lines<T, DIR, PER><<<(lp.nlines + 31) / 32, 32, 0, c->stream>>>(g, c->F<T>(), lp);
        note(c, 2);
        return false;
    }
    // mixed without a constant factorisation: the partitioned solve in
    // double, one thread per chunk of m rows
    k_tri_a<T, DIR, PER><<<(nt + 127) / 128, 128, 0, c->stream>>>(g, c->F<T>(), lp);
    note(c);
    k_tri_b<T, DIR, PER><<<(lp.nlines + 127) / 128, 128, 0, c->stream>>>(g, c->F<T>(), lp);
    note(c);
    k_tri_c<T, DIR><<<(nt + 127) / 128, 128, 0, c->stream>>>(g, c->F<T>(), lp);
    note(c);
    return false;
}

// ESTIMATE_HUV; with_post = false leaves the GET_Eta_U_V_HU_HV tail (k_post)
// to the fused kernel of the stage
template <typename T> static void launch_estimate_huv_opt(fw_ctx *c, int istage, bool with_post) {
    const Grid &g = c->g;
    static const double AL[3] = {0.0, 3.0 / 4.0, 1.0 / 3.0};
    static const double BE[3] = {1.0, 1.0 / 4.0, 2.0 / 3.0};
    const T al = (T)AL[istage - 1], be = (T)BE[istage - 1];
    // stage 2 too: with PERIODIC, EXCHANGE leaves the x-ghost values of the
    // previous exchange in the ghost corners (bc.F:735-740), so the last
    // stage's corners hold the second stage's values
    if (istage >= 2 && g.track_rad)
        k_update<T, true><<<grid2(g.Mloc, g.Nloc, c->blk(TK_UPDATE)), c->blk(TK_UPDATE), 0, c->stream>>>(
            g, c->F<T>(), al, be);
    else
        k_update<T><<<grid2(g.Mloc, g.Nloc, c->blk(TK_UPDATE)), c->blk(TK_UPDATE), 0, c->stream>>>(g, c->F<T>(), al,
                                                                                                     be);
    note(c);
    if (g.dispersion) {
        if (sizeof(T) == sizeof(float) && c->factored) {
            // factor both directions (when MASK9 changed) in one launch each,
            // then solve; the x solve resets the change flag when it can
            const int nbx = (c->px.nlines * c->px.P + 127) / 128;
            const int nby = (c->py.nlines * c->py.P + 127) / 128;
            const int lbx = (c->px.nlines + 127) / 128, lby = (c->py.nlines + 127) / 128;
            if (g.periodic) {
                k_fac_a_xy<T, true><<<nbx + nby, 128, 0, c->stream>>>(g, c->F<T>(), c->px, c->py, nbx);
                k_fac_b_xy<T, true><<<lbx + lby, 128, 0, c->stream>>>(g, c->F<T>(), c->px, c->py, lbx);
            } else {
                k_fac_a_xy<T, false><<<nbx + nby, 128, 0, c->stream>>>(g, c->F<T>(), c->px, c->py, nbx);
                k_fac_b_xy<T, false><<<lbx + lby, 128, 0, c->stream>>>(g, c->F<T>(), c->px, c->py, lbx);
            }
            note(c, 2);
            const bool cleared = launch_tri<T, 0, false>(c, c->px, false, true);
            if (g.periodic) launch_tri<T, 1, true>(c, c->py, false);
            else launch_tri<T, 1, false>(c, c->py, false);
            if (!cleared) {
                k_fac_clear<<<1, 1, 0, c->stream>>>(c->F<T>().m9_dirty);
                note(c);
            }
        } else {
            launch_tri<T, 0, false>(c, c->px);
            if (g.periodic) launch_tri<T, 1, true>(c, c->py);
            else launch_tri<T, 1, false>(c, c->py);
        }
    }
    if (!with_post) return;
    k_post<T><<<grid2(g.Mloc, g.Nloc, B2D), B2D, 0, c->stream>>>(g, c->F<T>());
    note(c);
    if (!g.dispersion) {
        k_nodisp_copy<T><<<grid2(g.Mloc, g.Nloc, B2D), B2D, 0, c->stream>>>(g, c->F<T>());
        note(c);
    }
}

template <typename T> void launch_estimate_huv(fw_ctx *c, int istage) { launch_estimate_huv_opt<T>(c, istage, true); }

template <typename T> void launch_update_mask(fw_ctx *c) {
    const Grid &g = c->g;
    k_mask<T><<<grid2(g.Mloc + 1, g.Nloc + 1, B2D), B2D, 0, c->stream>>>(g, c->F<T>());
    note(c);
    auto &F = c->F<T>();
    uint8_t *t = F.MASK;
    F.MASK = F.MASKn;
    F.MASKn = t;
}

template <typename T> void launch_breaking(fw_ctx *c) {
    const Grid &g = c->g;
    if (!g.show_breaking) return;
    k_break_a<T><<<grid2(g.Mloc, g.Nloc, B2D), B2D, 0, c->stream>>>(g, c->F<T>());
    note(c);
    k_break_b<T><<<1, 1024, 0, c->stream>>>(g, c->F<T>());
    note(c);
    auto &F = c->F<T>();
    T *t = F.AGE;
    F.AGE = F.AGEn;
    F.AGEn = t;
}

// CALCULATE_Cm_Sm (wavemaker.F:831-891) on the wavemaker band: one thread
// per (band cell, frequency) sums the Ntheta directional components
//   Cm/Sm = sum_kt D_gen(kf,kt) exp(-beta_gen(kf) ((I-Ibeg) DX - Xc)^2)
//           cos/sin(rlamda(kf,kt) (J-Jbeg) DY + phi1(kf,kt))
// in double, in the reference's order, and stores it in the field precision.
// i0, j0: I-Ibeg and J-Jbeg of the band's first cell.
template <typename T>
__global__ void __launch_bounds__(256) k_cm_sm(int bw, int bh, int mf, int mt, int i0, int j0, double DX,
                                               double DY, double xc, const double *__restrict__ tab, T *Cm,
                                               T *Sm) {
    const long long nb = (long long)bw * bh;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nb * mf) return;
    const int kf = (int)(t / nb);
    const long long b = t - (long long)kf * nb;
    const int bj = (int)(b / bw), bi = (int)(b - (long long)bj * bw);
    const double *dgen = tab, *rlamda = tab + (size_t)mf * mt, *phi = tab + 2 * (size_t)mf * mt;
    const double *betagen = tab + 3 * (size_t)mf * mt;
    const double dx = (double)(i0 + bi) * DX - xc;
    const double y = (double)(j0 + bj) * DY - 0.0;
    const double ex = exp(-betagen[kf] * (dx * dx));
    double cm = 0.0, sm = 0.0;
    for (int kt = 0; kt < mt; kt++) {
        const size_t k2 = (size_t)kf + (size_t)kt * mf;
        const double amp = dgen[k2] * ex;
        const double arg = rlamda[k2] * y + phi[k2];
        cm = cm + amp * cos(arg);
        sm = sm + amp * sin(arg);
    }
    Cm[b + (size_t)kf * nb] = (T)cm;
    Sm[b + (size_t)kf * nb] = (T)sm;
}

template <typename T>
void launch_cm_sm(fw_ctx *c, int bw, int bh, int i0, int j0, const double *tab, T *Cm, T *Sm) {
    const Grid &g = c->g;
    const long long n = (long long)bw * bh * g.nfreq;
    k_cm_sm<T><<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(bw, bh, g.nfreq, c->p.ntheta, i0, j0, g.DX,
                                                                   g.DY, g.xc_wk, tab, Cm, Sm);
    note(c);
}

template <typename T> void launch_end_step(fw_ctx *c) {
    const Grid &g = c->g;
    if (g.stats) {
        k_tsum<<<1, 1, 0, c->stream>>>(g, c->F<T>().dsc, c->F<T>().fsc);
        note(c);
    }
    k_end<T><<<grid2(g.Mloc, g.Nloc, B2D), B2D, 0, c->stream>>>(g, c->F<T>(), c->p.track_hmax);
    note(c);
    if (g.track_rad) {
        k_rad_derived<T><<<grid2(g.ie - g.ib + 1, g.je - g.jb + 1, B2D), B2D, 0, c->stream>>>(g, c->F<T>());
        note(c);
    }
}

template <typename T> void launch_stage(fw_ctx *c, int istage) {
    const Grid &g = c->g;
    if (g.dispersion) launch_dispersion<T>(c);
    launch_fluxes<T>(c);
    if (g.dispersion && g.show_breaking) {
        // GET_Eta_U_V_HU_HV tail + UPDATE_MASK + BREAKING (parallel part)
        // in one kernel, then the breaking sweep's candidates
        launch_estimate_huv_opt<T>(c, istage, false);
        k_post_mask_break<T><<<grid2(g.Mloc + 1, g.Nloc + 1, c->blk(TK_PMB)), c->blk(TK_PMB), 0, c->stream>>>(g, c->F<T>());
        note(c);
        auto &F = c->F<T>();
        uint8_t *t = F.MASK;
        F.MASK = F.MASKn;
        F.MASKn = t;
        k_break_b<T><<<1, 1024, 0, c->stream>>>(g, F);
        note(c);
        T *a = F.AGE;
        F.AGE = F.AGEn;
        F.AGEn = a;
    } else {
        launch_estimate_huv<T>(c, istage);
        launch_update_mask<T>(c);
        launch_breaking<T>(c);
    }
    launch_exchange<T>(c, g.direct_sponge != 0);
    if (istage >= 2 && g.track_rad) {
        const int n = 6 * g.Nglob + 6 * g.Mloc;
        k_ghost_rad<T><<<(n + 255) / 256, 256, 0, c->stream>>>(g, c->F<T>());
        note(c);
    }
}

#ifdef FW_SHARED_DEFS
// ---------------------------------------------------------------------------
// host-layout conversion: a Fortran (w x h, leading dimension w) array in a
// device staging buffer <-> a pitched field
// ---------------------------------------------------------------------------
template <typename S, typename D>
__global__ void k_unpack(const S *src, int w, int h, D *dst, int pitch) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= w || j >= h) return;
    dst[(size_t)i + (size_t)j * pitch] = (D)src[(size_t)i + (size_t)j * w];
}
template <typename S, typename D>
__global__ void k_pack(const S *src, int pitch, int w, int h, D *dst) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= w || j >= h) return;
    dst[(size_t)i + (size_t)j * w] = (D)src[(size_t)i + (size_t)j * pitch];
}
__global__ void k_unpack_mask(const int *src, int w, int h, uint8_t *dst, int pitch) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= w || j >= h) return;
    const int v = src[(size_t)i + (size_t)j * w];
    dst[(size_t)i + (size_t)j * pitch] = (uint8_t)(v > 0 ? 1 : 0);
}

void convert_in(fw_ctx *c, const void *staging, int is_mask, void *field, int w, int h) {
    const dim3 b(32, 8), gr((w + 31) / 32, (h + 7) / 8);
    if (is_mask) k_unpack_mask<<<gr, b, 0, c->stream>>>((const int *)staging, w, h, (uint8_t *)field, c->g.pitch);
    else k_unpack<double, float><<<gr, b, 0, c->stream>>>((const double *)staging, w, h, (float *)field, c->g.pitch);
    note(c);
}
void convert_out(fw_ctx *c, const void *field, int is_mask, void *staging, int w, int h) {
    const dim3 b(32, 8), gr((w + 31) / 32, (h + 7) / 8);
    if (is_mask) k_pack<uint8_t, int><<<gr, b, 0, c->stream>>>((const uint8_t *)field, c->g.pitch, w, h, (int *)staging);
    else k_pack<float, double><<<gr, b, 0, c->stream>>>((const float *)field, c->g.pitch, w, h, (double *)staging);
    note(c);
}

// float host arrays (an FP32 host's REAL(SP) fields) of the FP64 build:
// widened on the way in, rounded to nearest on the way out
void convert_in_f32(fw_ctx *c, const float *staging, double *field, int w, int h) {
    const dim3 b(32, 8), gr((w + 31) / 32, (h + 7) / 8);
    k_unpack<float, double><<<gr, b, 0, c->stream>>>(staging, w, h, field, c->g.pitch);
    note(c);
}
void convert_out_f32(fw_ctx *c, const double *field, float *staging, int w, int h) {
    const dim3 b(32, 8), gr((w + 31) / 32, (h + 7) / 8);
    k_pack<double, float><<<gr, b, 0, c->stream>>>(field, c->g.pitch, w, h, staging);
    note(c);
}

// values of one field at n cells (pitched offsets) as double; type 0 double,
// 1 float, 2 uint8 mask
__global__ void k_gather(const void *field, int type, const int *off, int n, double *out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int o = off[k];
    out[k] = type == 0 ? ((const double *)field)[o]
                       : type == 1 ? (double)((const float *)field)[o] : (double)((const uint8_t *)field)[o];
}
void gather_points(fw_ctx *c, const void *field, int type, const int *d_off, int n, double *d_out) {
    k_gather<<<(n + 127) / 128, 128, 0, c->stream>>>(field, type, d_off, n, d_out);
    note(c);
}

#endif  // FW_SHARED_DEFS

// one kernel of the step by name, for timing (fw_time_kernel)
template <typename T> int launch_by_name(fw_ctx *c, const char *name) {
    const Grid &g = c->g;
    Fields<T> &f = c->F<T>();
    const dim3 gc = grid2(g.Mloc, g.Nloc, B2D);
    auto is = [&](const char *n) { return std::strcmp(name, n) == 0; };
    if (is("disp_a")) k_disp_a<T><<<grid2(g.Mloc, g.Nloc, c->blk(TK_DISP_A)), c->blk(TK_DISP_A), 0, c->stream>>>(g, f);
    else if (is("disp_b")) k_disp_b<T><<<grid2(g.Mloc, g.Nloc, c->blk(TK_DISP_B)), c->blk(TK_DISP_B), 0, c->stream>>>(g, f);
    else if (is("flux_x")) { launch_flux<T, 0>(c); return 0; }
    else if (is("flux_y")) { launch_flux<T, 1>(c); return 0; }
    else if (is("update")) k_update<T><<<grid2(g.Mloc, g.Nloc, c->blk(TK_UPDATE)), c->blk(TK_UPDATE), 0, c->stream>>>(g, f, (T)0.75, (T)0.25);
    else if (is("post_mask_break")) {
        const dim3 b = c->blk(TK_PMB);
        k_post_mask_break<T><<<grid2(g.Mloc + 1, g.Nloc + 1, b), b, 0, c->stream>>>(g, f);
    }
    else if (is("tri_x")) { launch_tri<T, 0, false>(c, c->px); return 0; }
    else if (is("tri_y")) {
        if (g.periodic) launch_tri<T, 1, true>(c, c->py);
        else launch_tri<T, 1, false>(c, c->py);
        return 0;
    }
    else if (is("post")) k_post<T><<<gc, B2D, 0, c->stream>>>(g, f);
    else if (is("mask")) k_mask<T><<<grid2(g.Mloc + 1, g.Nloc + 1, B2D), B2D, 0, c->stream>>>(g, f);
    else if (is("break_a")) k_break_a<T><<<gc, B2D, 0, c->stream>>>(g, f);
    else if (is("ghost")) { launch_ghost<T>(c, g.visc_breaking != 0); return 0; }
    else if (is("maskmul")) k_maskmul<T><<<grid2(g.Mloc, g.Nloc, c->blk(TK_MASKMUL)), c->blk(TK_MASKMUL), 0, c->stream>>>(g, f, g.direct_sponge);
    else if (is("begin")) k_begin<T><<<gc, B2D, 0, c->stream>>>(g, f);
    else return -1;
    note(c);
    return 0;
}

#define INST(T)                                                  \
    template void launch_begin_step<T>(fw_ctx *);                \
    template void launch_exchange<T>(fw_ctx *, bool);            \
    template void launch_estimate_dt<T>(fw_ctx *);               \
    template void launch_dispersion<T>(fw_ctx *);                \
    template void launch_fluxes<T>(fw_ctx *);                    \
    template void launch_sources_debug<T>(fw_ctx *);             \
    template void launch_estimate_huv<T>(fw_ctx *, int);         \
    template void launch_update_mask<T>(fw_ctx *);               \
    template void launch_breaking<T>(fw_ctx *);                  \
    template void launch_sponge<T>(fw_ctx *);                    \
    template void launch_end_step<T>(fw_ctx *);                  \
    template void launch_stage<T>(fw_ctx *, int);     \
    template void launch_cm_sm<T>(fw_ctx *, int, int, int, int, const double *, T *, T *); \
    template int launch_by_name<T>(fw_ctx *, const char *);      \
    template bool flux_tma_attrs<T>();

}  // namespace fw
