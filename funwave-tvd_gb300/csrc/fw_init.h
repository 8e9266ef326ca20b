// fw_init.h -- host-side INITIALIZATION of a case (init.F:280-1272) and the
// wavemaker coefficients (wavemaker.F), computed in double on the host.
#pragma once

#include <string>
#include <vector>

#include "funwave_gpu.h"

namespace fw {

// Everything INITIALIZATION hands to the time loop, Fortran-ordered with
// ghost cells.  x-face arrays are (Mloc+1) x Nloc, y-face Mloc x (Nloc+1).
struct HostCase {
    int Mloc = 0, Nloc = 0;
    std::vector<double> Depth, Depthx, Depthy, Eta, U, V, H, HU, HV, Ubar, Vbar, Cd, SPONGE, nu;
    std::vector<int> MASK, MASK9, MASK_STRUC;
    double EtaBlowVal = 0, T_brk = 0;
    // WK_REG (wavemaker.F:2369-2405)
    double D_gen = 0, beta_gen = 0, rlamda = 0, Width_WK = 0;
    // wavemaker band, 1-based inclusive (init.F:1236-1268); empty if ilo > ihi
    int ilo = 0, ihi = -1, jlo = 0, jhi = -1;
    // JON_2D: omega_k and the spectrum tables the device turns into the band
    // Cm/Sm (CALCULATE_Cm_Sm runs as a kernel); phases phi1 (kf fastest)
    std::vector<double> omega;
    std::vector<double> jon_dgen, jon_rlamda, jon_betagen, jon_phases;  // (kf fastest)
};

// Returns FW_OK or FW_ERR_BAD_PARAM (err says why).
int build_case(const fw_params &p, const double *depth, const double *eta, const double *u, const double *v,
               const double *phases, HostCase &hc, std::string &err);

}  // namespace fw
