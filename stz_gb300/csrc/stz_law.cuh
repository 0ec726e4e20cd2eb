// The STZ plasticity laws and the adaptive plastic sub-stepping, templated on
// the scalar type: double in the time-step kernel, a dual number (value and
// six partial derivatives) in the adjoint, so that both evaluate the same
// expression sequence.
#pragma once

#include "step.cuh"

namespace stzg {

__host__ __device__ inline double value(double x) { return x; }

// Parameters the laws read; S is the type of the differentiable ones (c0,
// Omega*eps0, chi_inf, s_y).
template <typename S> struct stz_law_params {
    int stz_model, t_model, substep_cap;
    double t_scale, adapt_fac, theta, Delta, tau0, kappa, rho, mu;
    S c0, Omegaeps0, chi_inf, s_y;
};

__host__ __device__ inline stz_law_params<double> law_params(const step_consts &c) {
    stz_law_params<double> p;
    p.stz_model = c.stz_model;
    p.t_model = c.t_model;
    p.substep_cap = c.substep_cap;
    p.t_scale = c.t_scale;
    p.adapt_fac = c.adapt_fac;
    p.theta = c.theta;
    p.Delta = c.Delta;
    p.tau0 = c.tau0;
    p.kappa = c.kappa;
    p.rho = c.rho;
    p.mu = c.mu;
    p.c0 = c.c0;
    p.Omegaeps0 = c.Omegaeps0;
    p.chi_inf = c.chi_inf;
    p.s_y = c.s_y;
    return p;
}

// STZ plastic rate (stz_model.hh:9-207) with the yield stress s_y in place
// of the reference's unit s0 and `sbar<1`.
template <typename S>
__device__ __forceinline__ S dplastic(const stz_law_params<S> &c, S sbar, S chi, S &dchi1, S &dchi2) {
    const S s0 = c.s_y, Om = c.Omegaeps0;
    const double thetainv = 1 / c.theta, De = c.Delta, tau0 = c.tau0;
    if (c.stz_model == 0 || c.stz_model == 1) {
        S sC1, sC2, sC, sT;
        if (c.stz_model == 0) {  // stz_model.hh:58-67
            sC1 = exp(-De * thetainv);
            sC2 = cosh(Om * sbar * thetainv);
            sC = sC1 * sC2;
            sT = tanh(Om * sbar * thetainv);
        } else {  // stz_model.hh:76-87
            S x = Om * sbar / De;
            sC1 = exp(-De * thetainv);
            sC = exp(-De * cosh(x) * thetainv) * cosh(De * sinh(x) * thetainv);
            sC2 = sC / sC1;
            sT = tanh(De * sinh(x) * thetainv);
        }
        // Dplastic_common, stz_model.hh:30-48
        S sbart = value(sbar) > 1e-12 ? sbar : S(1e-12), bfac = exp(-1 / chi);
        S pM = 1 + sbart * sT / s0 + c.rho / (2 * sC2);
        S M = s0 / (2 * sbart) * (pM - sqrt(pM * pM - 4 * sbart * sT / s0));
        S Dpl = bfac * sC * (sT - M) / tau0;
        S Gamma = 2 * tau0 * Dpl * sbar / (s0 * bfac);
        bfac /= tau0 * c.c0;
        dchi1 = bfac * Gamma;
        dchi2 = bfac * c.kappa * sC1 * c.rho;
        return Dpl;
    }
    dchi2 = S(0);
    if (value(sbar) < value(s0)) {
        dchi1 = S(0);
        return S(0);
    }
    S sC, sT;
    if (c.stz_model == 3) {  // stz_model.hh:179-206
        S x = Om * sbar / De;
        sC = 0.5 * (exp(-De * thetainv * exp(x)) + exp(-De * thetainv * exp(-x)));
        sT = tanh(De * sinh(x) * thetainv);
    } else {  // stz_model.hh:103-151
        const int tm = c.t_model;
        if (tm == -1 || De >= value(Om * sbar)) {
            sC = 0.5 * (exp((Om * sbar - De) * thetainv) + exp((-Om * sbar - De) * thetainv));
        } else {
            S tmp;
            switch (tm) {
                case 0: sC = 0.5 * (exp((-Om * sbar - De) * thetainv) + 1); break;
                case 1: tmp = Om * sbar / De;
                        sC = 0.5 * (exp((-Om * sbar - De) * thetainv) + sqrt(0.5 * (1 + tmp * tmp))); break;
                case 2: tmp = Om * sbar / De;
                        sC = 0.5 * (exp((-Om * sbar - De) * thetainv) + (0.5 * (1 + tmp * tmp))); break;
                case 3: sC = sbar * (0.5 * Om / De); break;  // t_icpt=0, t_grad=Omegaeps0/(2 Delta)
                case 4: sC = 0.5 * (exp((-Om * sbar - De) * thetainv) + (Om * sbar - De) * thetainv + 1); break;
                default: sC = S(0);
            }
        }
        sT = tm != 3 ? tanh(Om * sbar * thetainv) : S(1);
    }
    S bfac = exp(-1 / chi);
    S Dpl = bfac * sC * (sT - s0 / sbar) / tau0;
    S Gamma = 2 * tau0 * Dpl * sbar / (s0 * bfac);
    dchi1 = bfac * Gamma / (tau0 * c.c0);
    return Dpl;
}

// shear_sim::adaptive_plastic_term, shear_sim.cc:513-548, with an iteration
// cap (the reference loop has none and never ends in stiff regimes).
template <typename S>
__device__ __forceinline__ S adaptive_plastic(const stz_law_params<S> &c, S sbar, S &chiv, S &ddev, double dt,
                                              int &iters) {
    const double theta_loc = 0;
    iters = 0;
    if (value(sbar) < 1e-12) {
        ddev = S(0);
        return S(0);
    }
    S dtl = S(dt), osbar = sbar, dplas, dchi1, dchi2, adt;
    bool adapt = true;
    do {
        dplas = 2 * c.t_scale * c.mu * dplastic(c, sbar, chiv, dchi1, dchi2);
        if (value(fabs(dtl * dplas)) > c.adapt_fac) {
            adt = c.adapt_fac / fabs(dplas);
            dtl -= adt;
        } else {
            adapt = false;
            adt = dtl;
        }
        sbar -= adt * dplas;
        chiv += (dchi1 * (c.chi_inf - chiv) + dchi2 * (theta_loc - chiv)) * c.t_scale * adt;
        if (++iters >= c.substep_cap) break;
    } while (adapt);
    ddev = osbar - sbar;
    return value(ddev) == 0 ? S(0) : ddev / osbar;
}


}  // namespace stzg
