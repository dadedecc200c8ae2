/*
 * ref_pin.c — host build of the reference's own pointwise functions, used
 * only to pin the oracle's restatement (test infrastructure).
 *
 * Compiled by oracle/build_oracle.py --ref with -I pointing at the
 * reference tree; the reference headers are included where they lie and
 * are not copied.  thermo_utils.h and phase_functions.h are header-only
 * `__device__ __host__` code, so defining the qualifiers away gives the
 * reference's exact host arithmetic.
 */
#define __device__
#define __host__
#define THERMO_UTILS_DEFINE_GLOBALS
#include <math.h>
#include <stddef.h>
#include "thermo_utils.h"
#include "phase_functions.h"

void ref_set_convex(int on) { h_thermo_convex_extrapolation_enabled = on; }
double ref_h(double p) { return h_of_phi(p); }
double ref_hp(double p) { return h_prime_of_phi(p); }
double ref_gp(double p) { return g_prime_of_phi(p); }
double ref_mu_A(double x, double T, double s) { return mu_A_dimless(x, T, s); }
double ref_mu_B(double x, double T, double s) { return mu_B_dimless(x, T, s); }
double ref_gamma(double x, double h, double Vm0, double dVm, double Vmc, double T, double s) {
    return gamma_thermo_nonlinear(x, h, Vm0, dVm, Vmc, T, s);
}
double ref_xB_eq(double T) { return xB_eq_from_temperature(T); }
double ref_sigmoid(double Y, double Yc, double eps) { return sigmoid_from_logit(Y, Yc, eps); }
double ref_logit(double x, double eps, double Yc) { return logit_from_fraction(x, eps, Yc); }
double ref_c_xB_phi(double x, double Vm0, double dVm, double Vmc, double h) {
    return c_xB_phi(x, Vm0, dVm, Vmc, h);
}
double ref_mu_tot_mix(double a, double b, double x, double m0, double h) {
    return mu_tot_mix(a, b, x, m0, h);
}
