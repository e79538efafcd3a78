// physical.cu -- behf_physical_gradient: the chain rule from the nine cell-centred moduli that the library works in
// (rho, rho_f, mu, M, C, H, lambda_u, b, m: the outputs of the reference's create_model_all, outputfunc.cpp:202-217)
// to Biot's physical parameters lambda (drained Lame), mu, rho, rho_f, M, alpha and kappa.  Host arithmetic only.
//
// The moduli as functions of the physical parameters, with the viscosity eta and the ratio m / rho_f =
// (1 + 2/8) tau / phi held fixed per cell (tortuosity and porosity are not inverted):
//     C = alpha M,   lambda_u = lambda + alpha^2 M,   H = lambda_u + 2 mu,   b = eta / kappa,   m = (m/rho_f) rho_f
// and rho, rho_f, mu, M themselves.  So, with g_X = dJ/dX:
//     g_lambda = g_H + g_lambda_u                       g_alpha = M g_C + 2 alpha M (g_H + g_lambda_u)
//     g_mu     = g_mu + 2 g_H                           g_kappa = -(eta / kappa^2) g_b = -(b^2 / eta) g_b
//     g_rho    = g_rho                                  g_rho_f = g_rho_f + (m / rho_f) g_m
//     g_M      = g_M + alpha g_C + alpha^2 (g_H + g_lambda_u)
// with alpha = C / M per cell.  Pure-fluid cells (mu = 0, b = 0, C = M) get alpha = 1 and g_kappa = 0.
#include <cmath>
#include <cstddef>

#include "behf.h"

namespace behf {
void report_error(const char* msg);
}

extern "C" behf_status behf_physical_gradient(long long ncell, const float* const moduli[BEHF_NMOD],
                                              const double* const grad_moduli[BEHF_NMOD], double eta,
                                              double* const grad_phys[BEHF_NPHYS]) {
    if (ncell < 0 || !moduli || !grad_moduli || !grad_phys || !(eta > 0)) {
        behf::report_error("behf_physical_gradient: bad argument (need ncell >= 0, eta > 0, non-null arrays)");
        return BEHF_ERR_INVALID;
    }
    const int need[] = {BEHF_RHOF, BEHF_M, BEHF_C, BEHF_C1, BEHF_C2};
    for (int q : need)
        if (!moduli[q]) {
            behf::report_error("behf_physical_gradient: moduli rho_f, M, C, b and m are required");
            return BEHF_ERR_INVALID;
        }
    const double* G[BEHF_NMOD];
    for (int q = 0; q < BEHF_NMOD; q++) G[q] = grad_moduli[q];
    for (long long c = 0; c < ncell; c++) {
        auto g = [&](int q) { return G[q] ? G[q][c] : 0.0; };
        const double M = moduli[BEHF_M][c], C = moduli[BEHF_C][c], b = moduli[BEHF_C1][c];
        const double rf = moduli[BEHF_RHOF][c], m = moduli[BEHF_C2][c];
        const double alpha = M != 0 ? C / M : 0.0;
        const double gl = g(BEHF_HH) + g(BEHF_H2U);
        const double out[BEHF_NPHYS] = {
            gl,                                              // lambda
            g(BEHF_MU) + 2.0 * g(BEHF_HH),                   // mu
            g(BEHF_RHO),                                     // rho
            g(BEHF_RHOF) + (rf != 0 ? m / rf : 0.0) * g(BEHF_C2),  // rho_f
            g(BEHF_M) + alpha * g(BEHF_C) + alpha * alpha * gl,    // M
            M * g(BEHF_C) + 2.0 * alpha * M * gl,            // alpha
            -(b * b / eta) * g(BEHF_C1),                     // kappa
        };
        for (int q = 0; q < BEHF_NPHYS; q++)
            if (grad_phys[q]) grad_phys[q][c] = out[q];
    }
    return BEHF_OK;
}
