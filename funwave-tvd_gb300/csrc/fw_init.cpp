// fw_init.cpp -- host-side INITIALIZATION (init.F:280-1272), direct sponge
// (sponge.F:591-767) and wavemaker synthesis (wavemaker.F:55-194, 370-413,
// 831-891, 2128-2405), in double.  Runs once per case on the host; its
// results are uploaded to the device by fw_init().
//
// Default-REAL literals of the reference's FP64 build are widened from
// float: pi (mod_param.F:71) and the WK_REG constants -0.39, 1./3., 3.14159
// (wavemaker.F:2378-2399).
#include "fw_init.h"

#include <cmath>
#include <cstring>

namespace fw {

namespace {

constexpr double PI_SP = (double)(float)3.141592653;
constexpr double GRAV = 9.81;
constexpr double SMALL = 0.000001;
constexpr double LARGE = 999999.0;
constexpr int NG = 3;

// a^n for integer n by squaring, as the Fortran run time evaluates x**n
double ipow(double x, int n) {
    double r = 1.0;
    bool neg = n < 0;
    unsigned u = neg ? (unsigned)(-n) : (unsigned)n;
    while (u) {
        if (u & 1u) r *= x;
        x *= x;
        u >>= 1;
    }
    return neg ? 1.0 / r : r;
}

struct View {
    std::vector<double> &a;
    int ld;
    double &operator()(int I, int J) { return a[(size_t)(I - 1) + (size_t)(J - 1) * ld]; }
};
struct IView {
    std::vector<int> &a;
    int ld;
    int &operator()(int I, int J) { return a[(size_t)(I - 1) + (size_t)(J - 1) * ld]; }
};

// PHI_COLL, VTYPE 1, serial (bc.F:631-844)
void fill_scalar(std::vector<double> &phi, int M, int N, bool periodic) {
    View P{phi, M};
    const int Ib = NG + 1, Ie = M - NG, Jb = NG + 1, Je = N - NG;
    if (periodic)
        for (int I = 1; I <= M; I++)
            for (int K = 1; K <= NG; K++) {
                P(I, K) = P(I, Je - NG + K);
                P(I, Je + K) = P(I, NG + K);
            }
    for (int J = Jb; J <= Je; J++)
        for (int K = 1; K <= NG; K++) {
            P(K, J) = P(Ib + NG - K, J);
            P(Ie + K, J) = P(Ie - K + 1, J);
        }
    if (!periodic)
        for (int I = 1; I <= M; I++)
            for (int K = 1; K <= NG; K++) {
                P(I, K) = P(I, Jb + NG - K);
                P(I, Je + K) = P(I, Je - K + 1);
            }
}

// WK_WAVEMAKER_REGULAR_WAVE (wavemaker.F:2369-2405)
void wk_regular(const fw_params &p, HostCase &hc) {
    const double theta = p.theta_wk * PI_SP / 180.0;
    const double alpha = (double)(float)-0.39;
    const double alpha1 = alpha + (double)(1.0f / 3.0f);
    const double omgn = 2.0 * PI_SP / p.tperiod;
    const double h = p.dep_wk;
    const double tb = omgn * omgn * h / GRAV;
    const double tc = 1.0 + tb * alpha;
    const double wkn = std::sqrt((tc - std::sqrt(tc * tc - 4.0 * alpha1 * tb)) / (2.0 * alpha1)) / h;
    const double C_phase = 1.0 / wkn / p.tperiod * 2.0 * PI_SP;
    const double L = C_phase * p.tperiod;
    hc.rlamda = wkn * std::sin(theta);
    hc.Width_WK = p.delta_wk * L / 2.0;
    hc.beta_gen = 80.0 / (p.delta_wk * p.delta_wk) / (L * L);
    const double rl = wkn * std::cos(theta);
    const double rI = std::sqrt((double)(float)3.14159 / hc.beta_gen) * std::exp(-(rl * rl) / 4.0 / hc.beta_gen);
    const double kh = wkn * h;
    hc.D_gen = 2.0 * p.amp_wk * std::cos(theta) * (omgn * omgn - alpha1 * GRAV * ipow(wkn, 4) * ipow(h, 3)) /
               (omgn * wkn * rI * (1.0 - alpha * (kh * kh)));
}

double jon_theta(const fw_params &p, int kt) {
    double th = -PI_SP / 3.0 + p.theta_peak * PI_SP / 180.0 +
                2.0 / 3.0 * PI_SP / ((double)(float)p.ntheta - 1.0) * ((double)(float)kt - 1.0);
    if (th > 0.5 * PI_SP) th = 0.5 * PI_SP;
    if (th < -0.5 * PI_SP) th = -0.5 * PI_SP;
    return th;
}

// WK_EQUAL_DFREQ_IRREGULAR_WAVE (wavemaker.F:2128-2357) with injected phases
void jon_spectrum(const fw_params &p, HostCase &hc) {
    const int mf = p.nfreq, mt = p.ntheta;
    const double h = p.dep_wk, fm = p.freq_peak, delta = p.delta_wk;
    std::vector<double> freq(mf), EB(mf), AG(mt);
    hc.omega.assign(mf, 0.0);
    hc.jon_dgen.assign((size_t)mf * mt, 0.0);
    hc.jon_rlamda.assign((size_t)mf * mt, 0.0);
    hc.jon_betagen.assign(mf, 0.0);
    const double df = (p.freq_max - p.freq_min) / (mf - 1.0);
    double Ef = 0.0;
    for (int k = 1; k <= mf; k++) {
        const double f = p.freq_min + (k - 1) * df;
        freq[k - 1] = f;
        const double sig = f > fm ? 0.09 : 0.07;
        const double r = f / fm - 1.0;
        const double E = GRAV * GRAV * ipow(f, -5) * ipow(2.0 * PI_SP, -4) * 1.0 * std::exp(-5.0 / 4.0 * ipow(f / fm, -4)) *
                         std::pow(p.gamma_tma, std::exp(-(r * r) / (2.0 * (sig * sig))));
        EB[k - 1] = E * df;
        Ef = Ef + EB[k - 1];
    }
    if (mt == 1) {
        AG[0] = 1.0;
    } else {
        double sum = 0.0;
        if (p.spreading == FW_SPREAD_COS2S) {
            for (int kt = 1; kt <= mt; kt++) {
                const double c = std::cos((jon_theta(p, kt) - p.theta_peak * PI_SP / 180.0) / 2.0);
                AG[kt - 1] = std::pow(std::fabs(c), 2.0 * p.spread_s);
                sum = sum + AG[kt - 1];
            }
        } else {
            const double st = p.sigma_theta * PI_SP / 180.0;
            const int nspec = (int)(20.0 / st);
            for (int kt = 1; kt <= mt; kt++) {
                const double th = jon_theta(p, kt);
                double ag = 1.0 / (2.0 * PI_SP);
                for (int kn = 1; kn <= nspec; kn++) {
                    const double a = (double)(float)kn * st;
                    ag = ag + (1.0 / PI_SP) * std::exp(-0.5 * (a * a)) * std::cos(kn * (th - p.theta_peak * PI_SP / 180.0));
                }
                AG[kt - 1] = ag;
                sum = sum + ag;
            }
        }
        for (int kt = 0; kt < mt; kt++) AG[kt] = std::fabs(AG[kt] / sum);
    }
    const double alpha_spec = p.hmo * p.hmo / 16.0 / Ef;
    const double alpha = -0.39, alpha1 = alpha + 1.0 / 3.0;
    double wave_length = 0.0;
    for (int kf = 1; kf <= mf; kf++)
        for (int kt = 1; kt <= mt; kt++) {
            const double Hmo_each = 4.0 * std::sqrt((alpha_spec * EB[kf - 1] * AG[kt - 1]));
            const double ap = Hmo_each / std::sqrt(2.0) / 2.0;
            double theta = (mt == 1) ? p.theta_peak * PI_SP / 180.0 : jon_theta(p, kt);
            const double omgn = 2.0 * PI_SP * freq[kf - 1];
            hc.omega[kf - 1] = omgn;
            const double tb = omgn * omgn * h / GRAV;
            const double tc = 1.0 + tb * alpha;
            double wkn = std::sqrt((tc - std::sqrt(tc * tc - 4.0 * alpha1 * tb)) / (2.0 * alpha1)) / h;
            if (wkn == 0.0) {
                wkn = SMALL;
                wave_length = std::sqrt(GRAV * h) / fm;
            } else {
                wave_length = (1.0 / wkn * fm * 2.0 * PI_SP) / fm;
            }
            if (p.periodic) {
                // direction snapped to a y-periodic wavenumber (wavemaker.F:2262-2296)
                double t1 = wkn, t2 = 0.0, t3 = 0.0;
                int I = 0;
                if (theta > 0.0) {
                    while (t3 < theta) {
                        I = I + 1;
                        t2 = I * 2.0 * PI_SP / p.DY / (p.Nglob - 1.0);
                        t3 = (t2 >= t1) ? PI_SP / 2.0 : std::asin(t2 / t1);
                    }
                    if (t2 < t1) t3 = std::asin((I - 1) * 2.0 * PI_SP / p.DY / (p.Nglob - 1.0) / t1);
                } else if (theta < 0.0) {
                    while (t3 > theta) {
                        I = I + 1;
                        t2 = I * 2.0 * PI_SP / p.DY / (p.Nglob - 1.0);
                        t3 = (t2 >= t1) ? -PI_SP / 2.0 : -std::asin(t2 / t1);
                    }
                    if (t2 < t1) t3 = -std::asin((I - 1) * 2.0 * PI_SP / p.DY / (p.Nglob - 1.0) / t1);
                }
                theta = t3;
            }
            const size_t k2 = (size_t)(kf - 1) + (size_t)(kt - 1) * mf;
            hc.jon_rlamda[k2] = wkn * std::sin(theta);
            const double bg = 80.0 / (delta * delta) / (wave_length * wave_length);
            hc.jon_betagen[kf - 1] = bg;
            const double rl = wkn * std::cos(theta);
            const double rI = std::sqrt(PI_SP / bg) * std::exp(-(rl * rl) / 4.0 / bg);
            const double kh = wkn * h;
            hc.jon_dgen[k2] = 2.0 * ap * std::cos(theta) * (omgn * omgn - alpha1 * GRAV * ipow(wkn, 4) * ipow(h, 3)) /
                              (omgn * wkn * rI * (1.0 - alpha * (kh * kh)));
        }
    hc.Width_WK = delta * wave_length / 2.0;
}

// CALCULATE_SPONGE (sponge.F:591-767), serial
void direct_sponge(const fw_params &p, HostCase &hc) {
    const int M = hc.Mloc, N = hc.Nloc;
    const size_t nc = (size_t)M * N;
    std::vector<double> t1(nc, 0.0), t2(nc, 0.0);
    View S{hc.SPONGE, M}, A1{t1, M}, A2{t2, M};
    const double R = p.r_sponge, A = p.a_sponge;
    const double floor_ = std::pow(A, ipow(R, 50));
    auto combine = [&]() {
        for (size_t k = 0; k < nc; k++) {
            hc.SPONGE[k] = t1[k] > t2[k] ? t1[k] : t2[k];
            if (hc.SPONGE[k] < floor_) hc.SPONGE[k] = 1.0;
        }
    };
    if (p.sponge_west > 0.0) {
        const int Iw = (int)(p.sponge_west / p.DX) + NG;
        for (int J = 1; J <= N; J++)
            for (int I = 1; I <= M; I++) {
                const double lim = S(I, J) > 1.0 ? S(I, J) : 1.0;
                const double ri = ipow(R, 50 * (I - 1) / (Iw - 1));
                const double a = std::pow(A, ri);
                A1(I, J) = a > lim ? a : lim;
            }
    }
    if (p.sponge_east > 0.0) {
        const int Iw = (int)(p.sponge_east / p.DX) + NG;
        for (int J = 1; J <= N; J++)
            for (int I = 1; I <= M; I++) {
                const double lim = S(I, J) > 1.0 ? S(I, J) : 1.0;
                const double ri = ipow(R, 50 * (M - I) / (Iw - 1));
                const double a = std::pow(A, ri);
                A2(I, J) = a > lim ? a : lim;
            }
    }
    combine();
    if (p.sponge_south > 0.0) {
        const int Iw = (int)(p.sponge_south / p.DY) + NG;
        for (int I = 1; I <= M; I++)
            for (int J = 1; J <= N; J++) {
                const double lim = S(I, J) > 1.0 ? S(I, J) : 1.0;
                const double ri = ipow(R, 50 * (J - 1) / (Iw - 1));
                const double a = std::pow(A, ri);
                A1(I, J) = a > lim ? a : lim;
            }
    }
    if (p.sponge_north > 0.0) {
        const int Iw = (int)(p.sponge_north / p.DY) + NG;
        for (int I = 1; I <= M; I++)
            for (int J = 1; J <= N; J++) {
                const double lim = S(I, J) > 1.0 ? S(I, J) : 1.0;
                const double ri = ipow(R, 50 * (N - J) / (Iw - 1));
                const double a = std::pow(A, ri);
                A2(I, J) = a > lim ? a : lim;
            }
    }
    combine();
}

}  // namespace

int build_case(const fw_params &p, const double *depth, const double *eta, const double *u, const double *v,
               const double *phases, HostCase &hc, std::string &err) {
    const int M = p.Mglob + 2 * NG, N = p.Nglob + 2 * NG, M1 = M + 1, N1 = N + 1;
    const int Ib = NG + 1, Ie = M - NG, Jb = NG + 1, Je = N - NG;
    const size_t nc = (size_t)M * N;
    if (!depth) {
        err = "depth is required";
        return FW_ERR_BAD_PARAM;
    }
    if (p.wavemaker == FW_WK_JON_2D && (!phases || p.nfreq < 2 || p.ntheta < 1)) {
        err = "JON_2D needs Nfreq >= 2, Ntheta >= 1 and the phases";
        return FW_ERR_BAD_PARAM;
    }
    hc.Mloc = M;
    hc.Nloc = N;
    hc.Depth.assign(nc, 10.0);  // init.F:549
    hc.Eta.assign(nc, 0.0);
    hc.U.assign(nc, 0.0);
    hc.V.assign(nc, 0.0);
    hc.H.assign(nc, 0.0);
    hc.HU.assign(nc, 0.0);
    hc.HV.assign(nc, 0.0);
    hc.Ubar.assign(nc, 0.0);
    hc.Vbar.assign(nc, 0.0);
    hc.Cd.assign(nc, p.cd_fixed);
    hc.SPONGE.assign(nc, 1.0);
    hc.nu.assign(nc, p.nu_bkg);
    hc.MASK.assign(nc, 1);
    hc.MASK9.assign(nc, 0);
    hc.MASK_STRUC.assign(nc, 1);
    hc.Depthx.assign((size_t)M1 * N, 0.0);
    hc.Depthy.assign((size_t)M * N1, 0.0);
    View D{hc.Depth, M}, E{hc.Eta, M}, Uv{hc.U, M}, Vv{hc.V, M};
    for (int J = Jb; J <= Je; J++)
        for (int I = Ib; I <= Ie; I++) {
            const size_t g = (size_t)(I - Ib) + (size_t)(J - Jb) * p.Mglob;
            D(I, J) = depth[g];
            if (eta) E(I, J) = eta[g];
            if (u) Uv(I, J) = u[g];
            if (v) Vv(I, J) = v[g];
        }
    fill_scalar(hc.Depth, M, N, p.periodic != 0);  // init.F:789-794
    // face depths (init.F:811-829)
    View DX_{hc.Depthx, M1}, DY_{hc.Depthy, M};
    for (int J = 1; J <= N; J++)
        for (int I = 2; I <= M; I++) DX_(I, J) = 0.5 * (D(I - 1, J) + D(I, J));
    for (int J = 1; J <= N; J++) {
        DX_(1, J) = 0.5 * (3.0 * D(1, J) - D(2, J));
        DX_(M1, J) = 0.5 * (3.0 * D(M, J) - D(M - 1, J));
    }
    for (int J = 2; J <= N; J++)
        for (int I = 1; I <= M; I++) DY_(I, J) = 0.5 * (D(I, J - 1) + D(I, J));
    for (int I = 1; I <= M; I++) {
        DY_(I, 1) = 0.5 * (3.0 * D(I, 1) - D(I, 2));
        DY_(I, N1) = 0.5 * (3.0 * D(I, N) - D(I, N - 1));
    }
    double mx = 0.0;  // init.F:847
    for (int J = Jb; J <= Je; J++)
        for (int I = Ib; I <= Ie; I++) mx = std::fmax(mx, std::fabs(D(I, J)));
    hc.EtaBlowVal = 100.0 * mx;
    // wavemaker (init.F:963)
    if (p.wavemaker == FW_WK_REG) {
        if (p.dep_wk == 0.0 || p.tperiod == 0.0) {
            err = "re-set depth, Tperiod for wavemaker";
            return FW_ERR_BAD_PARAM;
        }
        wk_regular(p, hc);
    } else if (p.wavemaker == FW_WK_JON_2D) {
        jon_spectrum(p, hc);
    }
    if (p.direct_sponge) direct_sponge(p, hc);
    // MASK and dry eta (init.F:1000-1014)
    IView MK{hc.MASK, M};
    for (int J = 1; J <= N; J++)
        for (int I = 1; I <= M; I++) {
            if (E(I, J) < -D(I, J)) {
                MK(I, J) = 0;
                E(I, J) = -p.min_depth - D(I, J);
            } else {
                MK(I, J) = 1;
            }
        }
    const double g3 = p.gamma3, mdf = p.min_depth_frc;
    for (size_t k = 0; k < nc; k++) {
        const double h = hc.Eta[k] * g3 + hc.Depth[k];
        hc.H[k] = h > mdf ? h : mdf;
        hc.HU[k] = hc.H[k] * hc.U[k];
        hc.HV[k] = hc.H[k] * hc.V[k];
    }
    // CAL_DISPERSION at initialisation runs before MASK9 exists (its value
    // is 0), so every dispersive term, and U1p, is zero there: Ubar = HU
    const double g1 = p.dispersion ? p.gamma1 : 0.0;
    for (size_t k = 0; k < nc; k++) {
        hc.Ubar[k] = hc.HU[k] + g1 * 0.0 * hc.H[k];
        hc.Vbar[k] = hc.HV[k] + g1 * 0.0 * hc.H[k];
    }
    for (size_t k = 0; k < nc; k++) {  // init.F:1106-1116
        if (hc.MASK_STRUC[k] == 0) hc.Depth[k] = -LARGE;
        hc.MASK[k] = hc.MASK[k] * hc.MASK_STRUC[k];
    }
    IView M9{hc.MASK9, M};  // init.F:1153-1159
    for (int J = Jb; J <= Je; J++)
        for (int I = Ib; I <= Ie; I++)
            M9(I, J) = MK(I, J) * MK(I - 1, J) * MK(I + 1, J) * MK(I + 1, J + 1) * MK(I, J + 1) * MK(I - 1, J + 1) *
                       MK(I + 1, J - 1) * MK(I, J - 1) * MK(I - 1, J - 1);
    for (int J = 2; J <= N - 1; J++)  // init.F:1210-1219
        for (int I = 2; I <= M - 1; I++)
            if (MK(I, J) < 1) {
                DX_(I, J) = D(I - 1, J);
                DX_(I + 1, J) = D(I + 1, J);
                DY_(I, J) = D(I, J - 1);
                DY_(I, J + 1) = D(I, J + 1);
            }
    hc.T_brk = p.show_breaking ? 20.0 : 0.0;  // init.F:1222-1224
    // wavemaker band (init.F:1236-1268)
    hc.ilo = Ie + 1;
    hc.ihi = Ib - 1;
    hc.jlo = Je + 1;
    hc.jhi = Jb - 1;
    for (int J = Jb; J <= Je; J++) {
        const double y = (J - Jb) * p.DY;
        if (std::fabs(y - p.yc_wk) < p.ywidth_wk / 2.0) {
            if (J < hc.jlo) hc.jlo = J;
            if (J > hc.jhi) hc.jhi = J;
        }
    }
    for (int I = Ib; I <= Ie; I++) {
        const double x = (I - Ib) * p.DX;
        if (std::fabs(x - p.xc_wk) < hc.Width_WK) {
            if (I < hc.ilo) hc.ilo = I;
            if (I > hc.ihi) hc.ihi = I;
        }
    }
    if (p.wavemaker == FW_WK_JON_2D) {
        const size_t n = (size_t)p.nfreq * p.ntheta;
        hc.jon_phases.assign(n, 0.0);
        if (phases) hc.jon_phases.assign(phases, phases + n);
    }
    return FW_OK;
}

}  // namespace fw
