/*
 * pf_oracle.h — CPU FP64 restatement of the CUDA_STO_PF time step.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle for the CUDA library in
 * cuda_sto_pf_gb300/: tests, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg may call it; the product path never does.
 *
 * It follows the reference driver sequence literally (main_cuda.cu:
 * 28427-31623): every dealias pass, clamp and normalisation in the order the
 * reference issues them, with the FFTs done by our own mixed-radix FP64
 * transform (the reference uses cuFFT, an un-vendored NVIDIA library; its
 * transform is the textbook unnormalised DFT, which this restates).
 *
 * Parity pinning: the thermodynamics and phase functions are checked against
 * the reference's own thermo_utils.h / phase_functions.h compiled on the
 * host (oracle/build_ref.sh -> oracle/_ref/libpfref.so) and against golden
 * vectors generated from them (tests/golden/), and the per-cell kernels of
 * the step against the reference's own cuda_kernels.cu built for the host
 * (oracle/ref_kernels.cpp -> oracle/_ref/librefk.so).  The step as a whole
 * is pinned by known-answer tests (Fourier-mode decay, homogeneous Eshelby
 * field, exact mass conservation) and, through the CUDA library it checks,
 * against the reference main_cuda rebuilt from its sources
 * (tests/test_ref_main_parity.py).
 */
#ifndef PF_ORACLE_H
#define PF_ORACLE_H

#include "../include/pfgb.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct pfo_state pfo_state;

/* derived thermo (pfparams_refresh_thermo, main_cuda.cu:15603-15613) */
void pfo_params_finalize(pfgb_params *p);

pfo_state *pfo_create(const pfgb_params *p);
void pfo_destroy(pfo_state *s);
int pfo_load_fields(pfo_state *s, const double *phi, const double *xB,
                    const double *eta, const double *dYdt_prev);
/* returns a pfgb_status code */
int pfo_step(pfo_state *s, int nsteps, pfgb_step_stats *stats);
/* test hooks: the step's phi / eta right-hand sides on given fields */
void pfo_test_phi_rhs(pfo_state *s, int coupling, const double *phi, const double *eta, const double *xB,
                      const double *sig, const double *eps, double *out);
void pfo_test_eta_rhs(pfo_state *s, const double *eta, const double *phi, const double *xB, const double *sig,
                      double *out);
void pfo_test_mu(pfo_state *s, const double *Y, const double *phiY, const double *sig, double *xB, double *mu);
void pfo_test_polarization(pfo_state *s, int lin, const double *phi, const double *eta, const double *xB,
                           const double *eps, double *out);
void pfo_test_green(pfo_state *s, const double *tau, double *u);
void pfo_test_dealias(pfo_state *s, double *k);
void pfo_test_xsplit_source(pfo_state *s, double mDx, const double *divJ, const double *phi_new,
                            const double *lap, double *rhs);
void pfo_test_xsplit_final(pfo_state *s, double dt, const double *x, const double *xB_old, double *Y, double *xB);
void pfo_test_flux(pfo_state *s, const double *g, const double *phiY, const double *etaY, const double *xB_prev,
                   double *J);
void pfo_test_cons_init(pfo_state *s, const double *phi, const double *xB, double *storage);
void pfo_test_cons_context(pfo_state *s, const double *storage, const double *phi, double *xB, double *Y);
long long pfo_test_cons_sweep(pfo_state *s, double *storage, const double *mu, const double *phi, const double *xB,
                              int axis, int parity, double spacing);
long long pfo_test_cons_constrain(pfo_state *s, double *phi_new, const double *phi_old, double *storage, double *xB,
                                  double *Y, long long *capped);
long long pfo_test_q_phase(pfo_state *s, const double *phi_new, const double *phi_old, const double *q_in,
                           double *q_out);
long long pfo_test_q_transport(pfo_state *s, double dt, const double *q_in, const double *divJ, const double *phi,
                               const double *xB_in, double *q_out, double *xB_out, double *Y_out);
void pfo_test_q_reconstruct(pfo_state *s, const double *q_in, const double *phi, const double *xB_in, double *q_out,
                            double *xB_out, double *Y_out);
void pfo_test_storage_exact(pfo_state *s, double dt, const double *divJ, const double *phi_new,
                            const double *phi_old, const double *Y_old, double *Y, double *xB);
void pfo_test_y_rhs(pfo_state *s, double dt, double mean_DY, const double *divJ, const double *phi_new,
                    const double *phi_old, const double *lapY, const double *Y, const double *dYdt, double *out);
/* GP storage coupling: the right-hand side with the GP storage source, the
 * storage point updates (Y_guess the Picard start), the eta feasibility pass
 * (returns the limited cells) and the <DY> sum */
void pfo_test_gp_y_rhs(pfo_state *s, double dt, double mean_DY, const double *divJ, const double *phi_new,
                       const double *phi_old, const double *eta_new, const double *eta_old, const double *lapY,
                       const double *Y, const double *dYdt, double *out);
void pfo_test_gp_storage(pfo_state *s, double dt, const double *divJ, const double *phi_new, const double *phi_old,
                         const double *eta_new, const double *eta_old, const double *Y_old, const double *Y_guess,
                         double *Y, double *xB);
long long pfo_test_gp_eta_feasibility(pfo_state *s, double dt, int limiter, double *eta, const double *eta_old,
                                      const double *phi_new, const double *phi_old, const double *xB_old,
                                      const double *divJ);
double pfo_test_gp_sum_dy(pfo_state *s, const double *phiY, const double *etaY, const double *Y);
/* minimize iterations (mode = minimize, full model, two_phase, zero mode off) */
int pfo_minimize(pfo_state *s, int max_iter, int stop_on_convergence, pfgb_min_stats *stats);
int pfo_read_fields(const pfo_state *s, double *phi, double *xB, double *Y,
                    double *eta, double *dYdt_prev);
int pfo_read_elastic(const pfo_state *s, double *sigma6, double *strain6);
int pfo_read_displacement_k(const pfo_state *s, double *u3);
int pfo_diagnostics(const pfo_state *s, pfgb_diag *d);
int pfo_set_threads(int n);
/* spectral bounds [a, b] of the elastic increment operator (elastic_chebyshev);
 * returns 0 when they are not below 1 */
int pfo_chebyshev_bounds(const double S[21], const double Sp[21], double *a, double *b);

/* FP64 3D transforms, cuFFT D2Z/Z2D conventions (unnormalised). */
void pfo_fft3d_r2c(int Nx, int Ny, int Nz, const double *in, double *out);
void pfo_fft3d_c2r(int Nx, int Ny, int Nz, const double *in, double *out);
/* 1D complex transform (sign=-1 forward), for FFT self-tests. */
void pfo_fft1d(int n, int sign, const double *in, double *out);

/* pointwise functions, exposed so tests can pin them against the
 * reference headers and golden vectors */
double pfo_h(double phi);
double pfo_hp(double phi);
double pfo_gp(double phi);
double pfo_mu_A(double xB, double T_K, double scale, int convex);
double pfo_mu_B(double xB, double T_K, double scale, int convex);
double pfo_gamma(double xB, double h, double Vm0, double dVm, double Vmc,
                 double T_K, double scale, int convex);
double pfo_xB_eq(double T_K);
double pfo_sigmoid(double Y, double Y_clip, double eps);
double pfo_logit(double xB, double eps, double Y_clip);
double pfo_meff(double Dm, double gamma);

#ifdef __cplusplus
}
#endif
#endif
