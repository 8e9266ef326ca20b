// fw_main.cpp -- a host driver with the shape of the reference's main
// program (src/main.F:45-575) over the C ABI of libfunwave_gpu.
//
//   fw_main [input.txt] [--dry-run]
//
// It reads input.txt with the reference's rules (READ_VALUE,
// mod_input.F:271-308: "KEY = value", "!" starts a comment, the first
// matching line wins), builds the depth as INITIALIZATION does for
// DEPTH_TYPE DATA / FLAT / SLOPE (init.F:684-760), creates and initialises
// the GPU context, then runs the time loop of main.F:284-535: OUTPUT at the
// top of every pass (io.F:52-134, PLOT_COUNT starting at PLOT_INTV so that
// the initial state is file 00001, init.F:631), one whole step per pass
// (fw_step), CHECK_BLOWUP's dump to file 99999 (misc.F:394-433).  PREVIEW
// (io.F:4304-4621) writes eta_NNNNN, u_NNNNN, v_NNNNN, mask_NNNNN (and
// hmax_NNNNN with OUT_Hmax, roller_NNNNN with ROLLER, U_undertow_NNNNN and
// V_undertow_NNNNN with UNDERTOW) in RESULT_FOLDER with PutFile's ASCII format
// (Mglob values per line, E16.6E4, interior only, io.F:4895-4921; or
// headerless binary with FIELD_IO_TYPE = BINARY), dep.out with the first
// file, and appends "TIME DT" to time_dt.out.  STATIONS writes sta_NNNN
// (time, eta, u, v per row, E21.10E4 and 3E16.5E4): unlike the reference,
// which drops the sample that finds its buffer full and pads the last
// buffer with TOTAL_TIME rows, every sample is kept and the last buffer
// holds only the rows taken.
//
// INI_UVZ starts from ETA_FILE / U_FILE / V_FILE at HotStartTime as the
// reference does; HOT_START / HOTSTART_FILE / HOTSTART_INTV restart from and
// write exact checkpoints (fw_checkpoint, fw_restore).
//
// --dry-run parses, builds the depth and writes dep.out without touching a
// GPU.  JON_2D phases, which the reference draws from the compiler's
// rand(0), come from SplitMix64 seeded by the key PHASE_SEED (default 1).
#include <algorithm>
#include <cctype>
#include <cinttypes>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <fstream>
#include <functional>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "funwave_gpu.h"

namespace {

constexpr double LARGE = 999999.0;
constexpr double TWO_PI = 6.283185307179586;

std::string upper(std::string s) {
    for (auto &ch : s) ch = (char)std::toupper((unsigned char)ch);
    return s;
}
std::string trim(const std::string &s) {
    size_t a = s.find_first_not_of(" \t\r\n'\""), b = s.find_last_not_of(" \t\r\n'\"");
    return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
}

// input.txt: key -> value text, first occurrence wins
struct Input {
    std::map<std::string, std::string> kv;
    bool load(const std::string &path) {
        std::ifstream f(path);
        if (!f) return false;
        std::string line;
        while (std::getline(f, line)) {
            const size_t bang = line.find('!');
            if (bang != std::string::npos) line = line.substr(0, bang);
            const size_t eq = line.find('=');
            if (eq == std::string::npos) continue;
            const std::string k = trim(line.substr(0, eq)), v = trim(line.substr(eq + 1));
            if (!k.empty() && !kv.count(k)) kv[k] = v;
        }
        return true;
    }
    bool has(const char *k) const { return kv.count(k) != 0; }
    std::string str(const char *k, const char *def) const { return has(k) ? kv.at(k) : std::string(def); }
    double num(const char *k, double def) const {
        if (!has(k)) return def;
        std::string v = kv.at(k);
        for (auto &ch : v)
            if (ch == 'd' || ch == 'D') ch = 'e';  // Fortran double exponent
        return std::strtod(v.c_str(), nullptr);
    }
    int flag(const char *k, int def) const {
        if (!has(k)) return def;
        const std::string u = upper(kv.at(k));
        const size_t p = u.find_first_not_of('.');
        return (p != std::string::npos && u[p] == 'T') ? 1 : 0;
    }
};

// an output switch: its input.txt key (e.g. "Hmax") or OUT_<key>
int out_flag(const Input &in, const char *key) {
    if (in.has(key)) return in.flag(key, 0);
    return in.flag((std::string("OUT_") + key).c_str(), 0);
}

// the input.txt keys of fw_params (names and defaults of src/io.F)
void fill_params(const Input &in, fw_params &p) {
    fw_params_default(&p);
    p.Mglob = (int)in.num("Mglob", 0);
    p.Nglob = (int)in.num("Nglob", 0);
    p.DX = in.num("DX", 0.0);
    p.DY = in.num("DY", 0.0);
    p.periodic = in.flag("PERIODIC", p.periodic);
    p.dispersion = in.flag("DISPERSION", p.dispersion);
    p.gamma1 = in.num("Gamma1", p.gamma1);
    p.gamma2 = in.num("Gamma2", p.gamma2);
    p.gamma3 = in.num("Gamma3", p.gamma3);
    p.beta_ref = in.num("Beta_ref", p.beta_ref);
    p.viscosity_breaking = in.flag("VISCOSITY_BREAKING", p.viscosity_breaking);
    p.show_breaking = in.flag("SHOW_BREAKING", p.show_breaking);
    p.cbrk1 = in.num("Cbrk1", p.cbrk1);
    p.cbrk2 = in.num("Cbrk2", p.cbrk2);
    p.wavemaker_cbrk = in.num("WAVEMAKER_Cbrk", p.wavemaker_cbrk);
    p.nu_bkg = in.num("nu_bkg", p.nu_bkg);
    p.swe_eta_dep = in.num("SWE_ETA_DEP", p.swe_eta_dep);
    p.cfl = in.num("CFL", p.cfl);
    if (in.has("DT_fixed")) {
        p.fixed_dt = 1;
        p.dt_fixed = in.num("DT_fixed", 0.0);
    }
    p.froude_cap = in.num("FroudeCap", p.froude_cap);
    p.min_depth = in.num("MinDepth", p.min_depth);
    p.min_depth_frc = in.num("MinDepthFrc", p.min_depth_frc);
    p.eta_limiter = in.flag("ETA_LIMITER", p.eta_limiter);
    p.trough_limit = in.num("TroughLimit", -LARGE);
    p.crest_limit = in.num("CrestLimit", LARGE);
    p.direct_sponge = in.flag("DIRECT_SPONGE", p.direct_sponge);
    p.sponge_west = in.num("Sponge_west_width", 0.0);
    p.sponge_east = in.num("Sponge_east_width", 0.0);
    p.sponge_south = in.num("Sponge_south_width", 0.0);
    p.sponge_north = in.num("Sponge_north_width", 0.0);
    p.r_sponge = in.num("R_sponge", p.r_sponge);
    p.a_sponge = in.num("A_sponge", p.a_sponge);
    p.friction_sponge = in.flag("FRICTION_SPONGE", p.friction_sponge);
    p.cd_fixed = in.num("Cd", 0.0);
    const std::string wk = upper(in.str("WAVEMAKER", "NONE"));
    p.wavemaker = wk.rfind("WK_REG", 0) == 0 ? FW_WK_REG : wk.rfind("JON_2D", 0) == 0 ? FW_WK_JON_2D : -1;
    if (wk == "NONE" || wk.empty()) p.wavemaker = FW_WK_NONE;
    p.amp_wk = in.num("AMP_WK", 0.0);
    p.tperiod = in.num("Tperiod", 0.0);
    p.dep_wk = in.num("DEP_WK", 0.0);
    p.xc_wk = in.num("Xc_WK", 0.0);
    p.yc_wk = in.num("Yc_WK", 0.0);
    p.theta_wk = in.num("Theta_WK", 0.0);
    p.delta_wk = in.num("Delta_WK", p.delta_wk);
    p.time_ramp = in.num("Time_ramp", 0.0);
    p.ywidth_wk = in.num("Ywidth_WK", LARGE);
    p.freq_peak = in.num("FreqPeak", 0.0);
    p.freq_min = in.num("FreqMin", 0.0);
    p.freq_max = in.num("FreqMax", 0.0);
    p.gamma_tma = in.num("GammaTMA", 3.3);
    p.hmo = in.num("Hmo", 0.0);
    p.theta_peak = in.num("ThetaPeak", 0.0);
    p.sigma_theta = in.num("Sigma_Theta", 10.0);
    p.nfreq = (int)in.num("Nfreq", 0);
    p.ntheta = (int)in.num("Ntheta", 1);
    p.spreading = upper(in.str("SPREADING", "WRAPPED_NORMAL")) == "COS2S" ? FW_SPREAD_COS2S : FW_SPREAD_WRAPPED_NORMAL;
    p.spread_s = in.num("SPREADING_S", 10.0);
    p.precision = upper(in.str("PRECISION", "FP64")) == "MIXED" ? FW_PREC_MIXED : FW_PREC_FP64;
    // the output switches under their input.txt keys (io.F:3392-3424), or
    // the OUT_* variable names
    p.track_hmax = out_flag(in, "Hmax");
    p.track_hmin = out_flag(in, "Hmin");
    p.track_umax = out_flag(in, "Umax");
    p.track_mfmax = out_flag(in, "MFmax");
    p.steady_time = in.num("STEADY_TIME", LARGE);
    p.t_intv_mean = in.num("T_INTV_mean", LARGE);
    p.track_roller = (in.flag("ROLLER", 0) || in.flag("UNDERTOW", 0)) ? 1 : 0;
    // PREVIEW_MEAN's Radiation files, and ulagm/vlagm of Umean/Vmean, need
    // CALCULATE_MEAN's radiation-stress sums
    p.track_radiation = (out_flag(in, "Radiation") || out_flag(in, "Umean") || out_flag(in, "Vmean")) ? 1 : 0;
}

// DEPTH_TYPE DATA / FLAT / SLOPE (init.F:684-760), interior Mglob x Nglob,
// column-major
// an interior Mglob x Nglob array as GetFile reads it: list-directed
// READ(1,*) row by row, Mglob values per J, J outer (init.F:1359-1379)
bool read_interior(const std::string &file, const fw_params &p, std::vector<double> &d, std::string &err) {
    const int M = p.Mglob, N = p.Nglob;
    d.assign((size_t)M * N, 0.0);
    std::ifstream f(file);
    if (!f) {
        err = file + " CANNOT BE FOUND";
        return false;
    }
    for (int j = 0; j < N; j++)
        for (int i = 0; i < M; i++) {
            std::string tok;
            if (!(f >> tok)) {
                err = "file " + file + " ends early";
                return false;
            }
            for (auto &ch : tok)
                if (ch == 'd' || ch == 'D') ch = 'e';
            d[(size_t)i + (size_t)j * M] = std::strtod(tok.c_str(), nullptr);
        }
    return true;
}

bool build_depth(const Input &in, const fw_params &p, std::vector<double> &d, std::string &err) {
    const int M = p.Mglob, N = p.Nglob;
    d.assign((size_t)M * N, 0.0);
    const std::string type = upper(in.str("DEPTH_TYPE", "DATA")).substr(0, 3);
    const double flat = in.num("DEPTH_FLAT", 10.0);
    if (type == "DAT") {
        if (!read_interior(in.str("DEPTH_FILE", "depth.txt"), p, d, err)) return false;
    } else if (type == "FLA") {
        for (auto &v : d) v = flat;
    } else if (type == "SLO") {
        const double slp = in.num("SLP", 0.0), xslp = in.num("Xslp", 0.0);
        const int i0 = (int)(xslp / p.DX) + 1;  // Fortran INT truncates
        for (int j = 0; j < N; j++)
            for (int I = 1; I <= M; I++)
                d[(size_t)(I - 1) + (size_t)j * M] = I >= i0 ? flat - slp * (I - i0) * p.DX : flat;
    } else {
        err = "DEPTH_TYPE " + type + " is not built";
        return false;
    }
    return true;
}

// Fortran Ew.dE4 of a value: 0.<d digits>E+eeee right-aligned in w
// characters (w <= 40, d <= 16)
void fortran_e4(double v, int w, int d, char *out) {
    char body[64], res[80];
    if (v == 0.0) {
        std::snprintf(body, sizeof body, "0.%0*dE+0000", d, 0);
    } else {
        char buf[64];
        std::snprintf(buf, sizeof buf, "%.*E", d - 1, v);  // m.mmmE+xx with d significant digits
        const bool neg = buf[0] == '-';
        const char *m = buf + (neg ? 1 : 0);
        const int e = std::atoi(std::strchr(m, 'E') + 1) + 1;
        char digits[24];
        int k = 0;
        for (const char *q = m; *q != 'E' && k < d; q++)
            if (*q != '.') digits[k++] = *q;
        digits[k] = 0;
        std::snprintf(body, sizeof body, "%s0.%sE%c%04d", neg ? "-" : "", digits, e < 0 ? '-' : '+', std::abs(e));
    }
    std::snprintf(res, sizeof res, "%*s", w, body);
    std::memcpy(out, res, (size_t)w);
    out[w] = 0;
}

// PutFile's ASCII line format: E16.6E4 of REAL(SP) values
void e16_6e4(float v, char *out) { fortran_e4((double)v, 16, 6, out); }

bool put_file(const std::string &path, const std::vector<double> &phi, const fw_params &p) {
    FILE *f = std::fopen(path.c_str(), "w");
    if (!f) return false;
    const int Mloc = p.Mglob + 6;
    char cell[17];
    for (int J = 4; J <= p.Nglob + 3; J++) {
        for (int I = 4; I <= p.Mglob + 3; I++) {
            e16_6e4((float)phi[(size_t)(I - 1) + (size_t)(J - 1) * Mloc], cell);
            std::fputs(cell, f);
        }
        std::fputc('\n', f);
    }
    return std::fclose(f) == 0;
}

// FIELD_IO_TYPE = BINARY (mod_parallel_field_io.F:161-221): the interior
// Mglob x Nglob in Fortran order, headerless, REAL(SP) of the build (double
// for FP64, float for MIXED), native byte order
bool put_file_binary(const std::string &path, const std::vector<double> &phi, const fw_params &p) {
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) return false;
    const int Mloc = p.Mglob + 6;
    for (int J = 4; J <= p.Nglob + 3; J++)
        for (int I = 4; I <= p.Mglob + 3; I++) {
            const double v = phi[(size_t)(I - 1) + (size_t)(J - 1) * Mloc];
            if (p.precision == FW_PREC_FP64) {
                std::fwrite(&v, sizeof v, 1, f);
            } else {
                const float fv = (float)v;
                std::fwrite(&fv, sizeof fv, 1, f);
            }
        }
    return std::fclose(f) == 0;
}

std::string numbered(const std::string &dir, const char *stem, int icount) {
    char b[16];
    std::snprintf(b, sizeof b, "%05d", icount % 100000);
    return dir + stem + "_" + b;
}

uint64_t splitmix64(uint64_t &s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

int fail(const char *what, int rc) {
    std::fprintf(stderr, "fw_main: %s: %s (%d)\n", what, fw_strerror(rc), rc);
    return 1;
}

}  // namespace

int main(int argc, char **argv) {
    std::string path = "input.txt";
    bool dry = false;
    for (int a = 1; a < argc; a++) {
        if (!std::strcmp(argv[a], "--dry-run")) dry = true;
        else path = argv[a];
    }
    Input in;
    if (!in.load(path)) {
        std::fprintf(stderr, "fw_main: cannot read %s\n", path.c_str());
        return 1;
    }
    fw_params p;
    fill_params(in, p);
    if (p.Mglob <= 0 || p.Nglob <= 0 || !(p.DX > 0) || !(p.DY > 0)) {
        std::fprintf(stderr, "fw_main: Mglob, Nglob, DX and DY are required\n");
        return 1;
    }
    if (p.wavemaker < 0) {
        std::fprintf(stderr, "fw_main: WAVEMAKER %s is not built\n", in.str("WAVEMAKER", "").c_str());
        return 1;
    }
    std::vector<double> depth;
    std::string err;
    if (!build_depth(in, p, depth, err)) {
        std::fprintf(stderr, "fw_main: %s\n", err.c_str());
        return 1;
    }
    const std::string dir = in.str("RESULT_FOLDER", "./output/");
    const double total = in.num("TOTAL_TIME", 0.0), plot_intv = in.num("PLOT_INTV", 1.0);
    const double plot_start = in.num("PLOT_START_TIME", 0.0);
    std::printf("fw_main: %d x %d, DX %g DY %g, %s, TOTAL_TIME %g, PLOT_INTV %g\n", p.Mglob, p.Nglob, p.DX, p.DY,
                p.precision == FW_PREC_MIXED ? "MIXED" : "FP64", total, plot_intv);

    const int Mloc = p.Mglob + 6, Nloc = p.Nglob + 6;
    std::vector<double> full((size_t)Mloc * Nloc, 0.0);
    // dep.out as PREVIEW writes it with the first file (interior of Depth)
    for (int j = 0; j < p.Nglob; j++)
        for (int i = 0; i < p.Mglob; i++) full[(size_t)(i + 3) + (size_t)(j + 3) * Mloc] = depth[(size_t)i + (size_t)j * p.Mglob];
    if (!put_file(dir + "dep.out", full, p)) {
        std::fprintf(stderr, "fw_main: cannot write to %s\n", dir.c_str());
        return 1;
    }
    if (dry) return 0;

    std::vector<double> phases;
    if (p.wavemaker == FW_WK_JON_2D) {
        uint64_t s = (uint64_t)in.num("PHASE_SEED", 1.0);
        phases.resize((size_t)p.nfreq * p.ntheta);
        for (auto &v : phases) v = (double)(splitmix64(s) >> 11) * (1.0 / 9007199254740992.0) * TWO_PI;
    }
    // INI_UVZ (io.F:712-801, init.F:1283-1386): the initial eta from
    // ETA_FILE and u, v from U_FILE and V_FILE (zero when V_FILE is not
    // given: the reference decides NO_UV_FILE by V_FILE alone), and TIME =
    // HotStartTime (main.F:188-190).  MASK_FILE is not read: the mask follows
    // from eta and depth (init.F:1000-1014, the NO_MASK_FILE rule).
    std::vector<double> eta0, u0, v0;
    const bool ini_uvz = in.flag("INI_UVZ", 0) != 0;
    if (ini_uvz) {
        if (in.flag("BED_DEFORMATION", 0)) {
            std::fprintf(stderr, "fw_main: BED_DEFORMATION is not built\n");
            return 1;
        }
        if (!in.has("ETA_FILE")) {
            std::fprintf(stderr, "fw_main: You use INI_UVZ, ETA_FILE NOT FOUND, STOP\n");
            return 1;
        }
        bool ok = read_interior(in.str("ETA_FILE", ""), p, eta0, err);
        if (ok && in.has("V_FILE"))
            ok = read_interior(in.str("U_FILE", ""), p, u0, err) && read_interior(in.str("V_FILE", ""), p, v0, err);
        if (!ok) {
            std::fprintf(stderr, "fw_main: %s\n", err.c_str());
            return 1;
        }
    }
    // exact checkpoints through fw_checkpoint / fw_restore, under the names
    // of the reference's declared hot-start variables (mod_global.F:141-145,
    // 387; main.F:73-133), which its input reader never sets:
    //   HOT_START = T     restore HOTSTART_FILE instead of initialising
    //   HOTSTART_INTV     every HOTSTART_INTV s of model time, write
    //                     RESULT_FOLDER/hotstart_NNNNN (NNNNN from 1)
    // Each checkpoint has a text companion <file>.host holding this driver's
    // output counters, so a restored run numbers and times its files as the
    // uninterrupted run would; station files are appended to.
    const bool hot_start = in.flag("HOT_START", 0) != 0;
    const std::string hot_file = in.str("HOTSTART_FILE", "");
    const double hot_intv = in.num("HOTSTART_INTV", 0.0);
    if (hot_start && hot_file.empty()) {
        std::fprintf(stderr, "fw_main: HOT_START needs HOTSTART_FILE\n");
        return 1;
    }
    fw_ctx *ctx = nullptr;
    int rc = fw_create(&p, &ctx);
    if (rc != FW_OK) return fail("fw_create", rc);
    if (hot_start) {
        rc = fw_restore(ctx, hot_file.c_str());
        if (rc != FW_OK) return fail("fw_restore", rc);
    } else {
        rc = fw_init(ctx, depth.data(), eta0.empty() ? nullptr : eta0.data(), u0.empty() ? nullptr : u0.data(),
                     v0.empty() ? nullptr : v0.data(), phases.empty() ? nullptr : phases.data());
        if (rc != FW_OK) return fail("fw_init", rc);
        if (ini_uvz && (rc = fw_set_scalar(ctx, "TIME", in.num("HotStartTime", 0.0))) != FW_OK)
            return fail("HotStartTime", rc);
    }

    FILE *tdt = std::fopen("time_dt.out", hot_start ? "a" : "w");
    int icount = 0;
    const bool binary = upper(in.str("FIELD_IO_TYPE", "ASCII")) == "BINARY";
    const bool out_roller = in.flag("ROLLER", 0) != 0, out_undertow = in.flag("UNDERTOW", 0) != 0;

    // STATIONS (io.F:3786-3954): grid indices from STATIONS_FILE, sampled
    // every PLOT_INTV_STATION into a buffer of StationOutputBuffer rows that
    // is written to sta_NNNN when full and at the end of the run
    const int nsta_req = (int)in.num("NumberStations", 0);
    const double plot_intv_sta = in.num("PLOT_INTV_STATION", 1.0);
    const int sta_buffer = std::max(1, (int)in.num("StationOutputBuffer", 1000));
    std::vector<int> sta_id, sta_i, sta_j;
    std::vector<FILE *> sta_f;
    std::vector<std::vector<double>> sta_rows;
    if (nsta_req > 0) {
        std::ifstream sf(in.str("STATIONS_FILE", "stations.txt"));
        if (!sf) {
            std::fprintf(stderr, "fw_main: %s THE STATION FILE CANNOT BE FOUND\n", in.str("STATIONS_FILE", "").c_str());
            return 1;
        }
        for (int k = 1; k <= nsta_req; k++) {
            double d1 = 0, d2 = 0;
            if (!(sf >> d1 >> d2)) break;
            const int is = (int)(3 + d1), js = (int)(3 + d2);  // Nghost + index, INTEGER assignment truncates
            if (is >= 4 && is <= p.Mglob + 3 && js >= 4 && js <= p.Nglob + 3) {
                char b[16];
                std::snprintf(b, sizeof b, "%04d", k);
                FILE *f = std::fopen((dir + "sta_" + b).c_str(), hot_start ? "a" : "w");
                if (!f) return 1;
                sta_id.push_back(k);
                sta_i.push_back(is);
                sta_j.push_back(js);
                sta_f.push_back(f);
                sta_rows.emplace_back();
            }
        }
    }
    auto flush_station = [&](size_t s) {
        char a[48], b[48];
        for (size_t r = 0; r + 4 <= sta_rows[s].size(); r += 4) {
            fortran_e4(sta_rows[s][r], 21, 10, a);
            std::fputs(a, sta_f[s]);
            for (int q = 1; q < 4; q++) {
                fortran_e4(sta_rows[s][r + q], 16, 5, b);
                std::fputs(b, sta_f[s]);
            }
            std::fputc('\n', sta_f[s]);
        }
        sta_rows[s].clear();
    };
    auto stations = [&](double t) -> int {
        const int n = (int)sta_i.size();
        if (n == 0) return FW_OK;
        std::vector<double> e(n), u(n), v(n), m(n);
        int r = fw_get_points(ctx, "Eta", n, sta_i.data(), sta_j.data(), e.data());
        if (r == FW_OK) r = fw_get_points(ctx, "U", n, sta_i.data(), sta_j.data(), u.data());
        if (r == FW_OK) r = fw_get_points(ctx, "V", n, sta_i.data(), sta_j.data(), v.data());
        if (r == FW_OK) r = fw_get_points(ctx, "MASK", n, sta_i.data(), sta_j.data(), m.data());
        if (r != FW_OK) return r;
        for (int s2 = 0; s2 < n; s2++) {
            const bool dry = m[s2] < 1.0;  // zeros on dry cells
            sta_rows[s2].insert(sta_rows[s2].end(), {t, dry ? 0.0 : e[s2], dry ? 0.0 : u[s2], dry ? 0.0 : v[s2]});
            if ((int)sta_rows[s2].size() / 4 >= sta_buffer) flush_station((size_t)s2);
        }
        return FW_OK;
    };
    // PREVIEW's fields, staged asynchronously (fw_output_begin): a snapshot
    // goes to one of two sets of pinned host buffers while the time loop
    // goes on; a writer thread formats and writes each set once its copies
    // are done, so neither the copies nor the formatting hold the steps
    std::vector<const char *> out_names = {"Eta", "U", "V", "MASK"};
    std::vector<std::string> out_stems = {"eta", "u", "v", "mask"};
    if (p.track_hmax) {
        out_names.push_back("HeightMax");
        out_stems.push_back("hmax");
    }
    if (out_roller) {  // io.F:4461-4471: roller_NNNNN, U_undertow_NNNNN, V_undertow_NNNNN
        out_names.push_back("ROLLER_FLUX");
        out_stems.push_back("roller");
    }
    if (out_undertow) {
        out_names.push_back("UNDERTOW_U");
        out_stems.push_back("U_undertow");
        out_names.push_back("UNDERTOW_V");
        out_stems.push_back("V_undertow");
    }
    const size_t nout = out_names.size(), plane = (size_t)Mloc * Nloc;
    struct OutSet {
        std::vector<void *> buf;
        int number = 0;
        bool busy = false;  // between fw_output_begin and the end of its writing
    } sets[2];
    for (auto &st : sets)
        for (size_t k = 0; k < nout; k++) {
            void *b = nullptr;
            const bool is_mask = out_stems[k] == "mask";
            if ((rc = fw_host_alloc(plane * (is_mask ? sizeof(int) : sizeof(double)), &b)) != FW_OK)
                return fail("fw_host_alloc", rc);
            st.buf.push_back(b);
        }
    std::mutex mu;
    std::condition_variable cv;
    std::deque<int> ready;  // sets whose copies are done, in order
    bool stop = false, write_failed = false;
    std::thread writer([&]() {
        std::vector<double> w(plane);
        for (;;) {
            int k;
            {
                std::unique_lock<std::mutex> lk(mu);
                cv.wait(lk, [&] { return stop || !ready.empty(); });
                if (ready.empty()) return;
                k = ready.front();
                ready.pop_front();
            }
            OutSet &st = sets[k];
            bool ok = true;
            for (size_t f = 0; f < nout; f++) {
                if (out_stems[f] == "mask") {
                    const int *m = (const int *)st.buf[f];
                    for (size_t q = 0; q < plane; q++) w[q] = m[q];
                } else {
                    std::memcpy(w.data(), st.buf[f], plane * sizeof(double));
                }
                const std::string path = numbered(dir, out_stems[f].c_str(), st.number);
                ok = (binary ? put_file_binary(path, w, p) : put_file(path, w, p)) && ok;
            }
            {
                std::lock_guard<std::mutex> lk(mu);
                st.busy = false;
                if (!ok) write_failed = true;
            }
            cv.notify_all();
        }
    });
    // on an early return the writer is stopped and joined (the files of
    // the snapshots already handed to it are written first)
    struct WriterGuard {
        std::function<void()> f;
        ~WriterGuard() { f(); }
    } writer_guard{[&] {
        if (!writer.joinable()) return;
        {
            std::lock_guard<std::mutex> lk(mu);
            stop = true;
        }
        cv.notify_all();
        writer.join();
    }};
    int in_flight = -1;  // the set whose copies may still run
    int next_set = 0;
    // hand the in-flight set to the writer once its copies are done
    auto collect = [&](bool wait) -> int {
        if (in_flight < 0) return FW_OK;
        if (wait) {
            const int r = fw_output_wait(ctx);
            if (r != FW_OK) return r;
        } else {
            const int d = fw_output_done(ctx);
            if (d < 0) return d;
            if (d == 0) return FW_OK;
        }
        {
            std::lock_guard<std::mutex> lk(mu);
            ready.push_back(in_flight);
        }
        cv.notify_all();
        in_flight = -1;
        return FW_OK;
    };
    // every snapshot taken so far written to its files
    auto drain = [&]() -> int {
        const int r = collect(true);
        std::unique_lock<std::mutex> lk(mu);
        cv.wait(lk, [&] { return ready.empty() && !sets[0].busy && !sets[1].busy; });
        if (r != FW_OK) return r;
        return write_failed ? FW_ERR_IO : FW_OK;
    };
    auto preview = [&](int number) -> int {
        icount = number;
        double t = 0.0, dt = 0.0;
        fw_get_scalar(ctx, "TIME", &t);
        fw_get_scalar(ctx, "DT", &dt);
        std::printf("PRINTING FILE NO. %5d TIME/TOTAL: %12.3f / %12.3f\n", icount, t, total);
        if (tdt) std::fprintf(tdt, "%.9E %.9E\n", t, dt);
        int r = collect(true);
        if (r != FW_OK) return r;
        OutSet &st = sets[next_set];
        {
            std::unique_lock<std::mutex> lk(mu);
            cv.wait(lk, [&] { return !st.busy; });
            if (write_failed) return FW_ERR_IO;
        }
        st.number = number;
        st.busy = true;
        r = fw_output_begin(ctx, (int)nout, out_names.data(), st.buf.data());
        if (r != FW_OK) {
            std::lock_guard<std::mutex> lk(mu);
            st.busy = false;
            return r;
        }
        in_flight = next_set;
        next_set ^= 1;
        return FW_OK;
    };
    auto finish_output = [&]() -> int {
        const int r = drain();
        {
            std::lock_guard<std::mutex> lk(mu);
            stop = true;
        }
        cv.notify_all();
        writer.join();
        for (auto &st : sets)
            for (void *b : st.buf) fw_host_free(b);
        return r;
    };

    // PREVIEW_MEAN (io.F:4630-4736): at the end of each CALCULATE_MEAN
    // interval, the means under RESULT_FOLDER/<stem>_NNNNN (NNNNN counts
    // the intervals); Sxx and Syy add 0.5*9.8*ETA2mean (default REAL)
    const bool o_umean = out_flag(in, "Umean"), o_vmean = out_flag(in, "Vmean");
    const bool o_etamean = out_flag(in, "ETAmean"), o_wh = out_flag(in, "WaveHeight");
    const bool o_rad = out_flag(in, "Radiation");
    const bool any_mean = p.steady_time < LARGE && (o_umean || o_vmean || o_etamean || o_wh || o_rad);
    double icount_mean = 0.0;
    std::vector<double> dep_full, etam, a, b;
    auto preview_mean = [&](int number) -> int {
        std::printf("  PRINTING MEAN FILE%6d\n", number);
        int r = FW_OK;
        auto get = [&](const char *name, std::vector<double> &v) {
            v.resize(plane);
            if (r == FW_OK) r = fw_get_field(ctx, name, v.data());
        };
        auto put = [&](const char *stem, const std::vector<double> &v) {
            if (r != FW_OK) return;
            const std::string path = numbered(dir, stem, number);
            if (!(binary ? put_file_binary(path, v, p) : put_file(path, v, p))) r = FW_ERR_IO;
        };
        if (dep_full.empty()) get("Depth", dep_full);
        get("ETAmean", etam);
        auto lagm = [&](const char *mean, const char *flux, const char *s1, const char *s2) {
            get(mean, a);
            put(s1, a);
            get(flux, b);
            for (size_t q = 0; q < plane; q++) b[q] = b[q] / std::max(dep_full[q] + etam[q], p.min_depth_frc);
            put(s2, b);
        };
        if (o_umean) lagm("Umean", "P_mean", "umean", "ulagm");
        if (o_vmean) lagm("Vmean", "Q_mean", "vmean", "vlagm");
        if (o_etamean) put("etamean", etam);
        if (o_wh) {
            get("WaveHeightRMS", a);
            put("Hrms", a);
            get("WaveHeightAve", a);
            put("Havg", a);
            get("SigWaveHeight", a);
            put("Hsig", a);
        }
        if (o_rad) {
            const double c49 = (double)(0.5f * 9.8f);
            std::vector<double> e2, ww;
            get("ETA2mean", e2);
            get("WWmean", ww);
            get("UUmean", a);
            for (size_t q = 0; q < plane && r == FW_OK; q++) a[q] = a[q] - ww[q] + c49 * e2[q];
            put("Sxx", a);
            get("UVmean", a);
            put("Sxy", a);
            get("VVmean", a);
            for (size_t q = 0; q < plane && r == FW_OK; q++) a[q] = a[q] - ww[q] + c49 * e2[q];
            put("Syy", a);
            const char *const names[][2] = {{"DxSxx", "DxSxx"}, {"DySxy", "DySxy"}, {"DySyy", "DySyy"},
                                            {"DxSxy", "DxSxy"}, {"PgrdX", "PgrdX"}, {"PgrdY", "PgrdY"},
                                            {"DxUUH", "DxUUH"}, {"DyUVH", "DyUVH"}, {"DyVVH", "DyVVH"},
                                            {"DxUVH", "DxUVH"}, {"FRCXmean", "FRCX"}, {"FRCYmean", "FRCY"},
                                            {"BreakDissX", "BrkDissX"}, {"BreakDissY", "BrkDissY"}};
            for (auto &nm : names) {
                get(nm[0], a);
                put(nm[1], a);
            }
        }
        return r;
    };

    double time = 0.0, dt = 0.0, plot_count = plot_intv;  // init.F:631
    double plot_count_sta = plot_intv_sta;                  // init.F:632
    double hot_count = 0.0;
    int hot_number = 0;
    fw_get_scalar(ctx, "TIME", &time);
    if (any_mean) fw_get_scalar(ctx, "ICOUNT_MEAN", &icount_mean);  // nonzero after a hot start
    if (hot_start) {
        // the counters the checkpointing run had (TIME and DT are restored)
        FILE *hf = std::fopen((hot_file + ".host").c_str(), "r");
        if (!hf || std::fscanf(hf, "%d %la %la %la %d", &icount, &plot_count, &plot_count_sta, &hot_count,
                               &hot_number) != 5) {
            std::fprintf(stderr, "fw_main: cannot read %s.host\n", hot_file.c_str());
            if (hf) std::fclose(hf);
            return 1;
        }
        std::fclose(hf);
        fw_get_scalar(ctx, "DT", &dt);
    }
    // a checkpoint at the top of a pass, after that pass's output; the
    // station rows taken so far are written first
    auto hotstart = [&]() -> int {
        int r = drain();
        if (r != FW_OK) return r;
        for (size_t k = 0; k < sta_f.size(); k++) {
            flush_station(k);
            std::fflush(sta_f[k]);
        }
        if (tdt) std::fflush(tdt);
        char b[16];
        std::snprintf(b, sizeof b, "%05d", ++hot_number);
        const std::string f = dir + "hotstart_" + b;
        r = fw_checkpoint(ctx, f.c_str());
        if (r != FW_OK) return r;
        FILE *hf = std::fopen((f + ".host").c_str(), "w");
        if (!hf) return FW_ERR_IO;
        std::fprintf(hf, "%d %a %a %a %d\n", icount, plot_count, plot_count_sta, hot_count, hot_number);
        return std::fclose(hf) == 0 ? FW_OK : FW_ERR_IO;
    };
    // a restored run begins at the step of the pass its checkpoint was
    // written in: that pass's output and counters are already done
    bool resume = hot_start;
    while (time < total) {  // DO WHILE (TIME < TOTAL_TIME)
        // OUTPUT (io.F:52-134) at the top of the pass, with the last DT
        if (!resume && !sta_i.empty()) {
            plot_count_sta += dt;
            if (plot_count_sta >= plot_intv_sta) {
                plot_count_sta -= plot_intv_sta;
                if ((rc = stations(time)) != FW_OK) return fail("STATIONS", rc);
            }
        }
        if (!resume && time >= plot_start) {
            plot_count += dt;
            if (plot_count >= plot_intv) {
                plot_count -= plot_intv;
                if ((rc = preview(icount + 1)) != FW_OK) return fail("PREVIEW", rc);
            }
        }
        if (!resume && hot_intv > 0.0) {
            hot_count += dt;
            if (hot_count >= hot_intv) {
                hot_count -= hot_intv;
                if ((rc = hotstart()) != FW_OK) return fail("fw_checkpoint", rc);
            }
        }
        resume = false;
        int status = FW_OK;
        rc = fw_step(ctx, 1, &status);
        if (rc != FW_OK) return fail("fw_step", rc);
        if (status != FW_OK) {
            // CHECK_BLOWUP: dump the state as file 99999, then stop
            std::fprintf(stderr, "fw_main: %s, dumping file 99999\n", fw_strerror(status));
            preview(99999);
            finish_output();
            fw_destroy(ctx);
            return 2;
        }
        if ((rc = collect(false)) != FW_OK) return fail("fw_output_done", rc);
        fw_get_scalar(ctx, "TIME", &time);
        fw_get_scalar(ctx, "DT", &dt);
        if (any_mean) {
            double n = 0.0;
            fw_get_scalar(ctx, "ICOUNT_MEAN", &n);
            if (n > icount_mean) {
                icount_mean = n;
                if ((rc = preview_mean((int)n)) != FW_OK) return fail("PREVIEW_MEAN", rc);
            }
        }
    }
    if ((rc = finish_output()) != FW_OK) return fail("output", rc);
    if (tdt) std::fclose(tdt);
    for (size_t k = 0; k < sta_f.size(); k++) {
        flush_station(k);
        std::fclose(sta_f[k]);
    }
    rc = fw_destroy(ctx);
    std::printf("fw_main: done, TIME %.6f, %d files\n", time, icount);
    return rc == FW_OK ? 0 : 1;
}
