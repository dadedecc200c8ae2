// ref_kernels.cpp — host build of the reference's own per-cell kernels
// (cuda_kernels.cu, the kernel section before its launch wrappers), used
// only to pin the oracle's restatement of the step.  Test infrastructure.
//
// oracle/build_oracle.py (build_ref_kernels) writes the kernel section of
// the reference's cuda_kernels.cu, as it lies in the reference tree, to
// oracle/_ref/ref_kernels_section.inc and compiles this file with the
// reference tree on the include path.  The CUDA qualifiers are defined
// away, the few device intrinsics the section names get host stand-ins, and
// a launch is a loop over the flat index: every kernel used here is one
// thread per cell, so the loop gives the kernel's exact arithmetic.
#include <cuda_runtime.h>
#include <cuComplex.h>
#include <cufft.h>
#include <vector_types.h>

#include <cmath>
#include <cstdint>
#include <cstring>

#undef __global__
#undef __device__
#undef __host__
#undef __forceinline__
#undef __constant__
#undef __shared__
#define __global__
#define __device__
#define __host__
#define __forceinline__ inline
#define __constant__
#define __shared__
#define THERMO_UTILS_DEFINE_GLOBALS

static uint3 threadIdx, blockIdx;
static dim3 blockDim, gridDim;
static inline void __syncthreads() {}
template <typename T> static inline T atomicAdd(T *a, T v) {
    const T o = *a;
    *a = o + v;
    return o;
}
static inline unsigned long long atomicCAS(unsigned long long *a, unsigned long long cmp, unsigned long long v) {
    const unsigned long long o = *a;
    if (o == cmp) *a = v;
    return o;
}
template <typename T> static inline T atomicExch(T *a, T v) {
    const T o = *a;
    *a = v;
    return o;
}
static inline long long __double_as_longlong(double d) {
    long long r;
    std::memcpy(&r, &d, sizeof(r));
    return r;
}
static inline double __longlong_as_double(long long l) {
    double r;
    std::memcpy(&r, &l, sizeof(r));
    return r;
}

#include "thermo_utils.h"
#include "phase_functions.h"
#include "pf_params.h"
#include "cuda_common.h"
#include "cuda_kernels.h"

// the dynamic shared arrays the section's reduction kernels declare extern
// (those kernels are compiled, never called here)
double sdata[1];
double pair_sdata[1];

#include "ref_kernels_section.inc"

// a launch of a one-thread-per-cell kernel over n cells
#define REF_LAUNCH(n, call)                                          \
    do {                                                             \
        blockDim.x = 1; blockDim.y = 1; blockDim.z = 1;              \
        gridDim.x = (unsigned)(n); gridDim.y = 1; gridDim.z = 1;     \
        threadIdx.x = 0; threadIdx.y = 0; threadIdx.z = 0;           \
        for (long long i_ = 0; i_ < (long long)(n); ++i_) {          \
            blockIdx.x = (unsigned)i_; blockIdx.y = 0; blockIdx.z = 0; \
            call;                                                    \
        }                                                            \
    } while (0)

extern "C" {

void refk_set_convex(int on) { h_thermo_convex_extrapolation_enabled = on; }

// compute_phi_rhs_kernel over n cells.  sig / eps: 6 n floats each, Voigt
// order xx yy zz yz xz xy (tensor strain); Sp: the 21 entries S_p_11 ..
// S_p_66; e00: xx yy zz yz xz xy.  d: T_K, mu_reference_scale, v_A, v_B,
// mu0_compound, Vm_compound, Vm_alpha_0, dVm_alpha_dxB, W, eps_iso_over_vB,
// gp_eps_iso, gp_elastic_derivative_scale, elastic_shift_dimless.
// i: gp_mode_enabled, gp_elastic_enabled, gp_elastic_active_phi,
// disable_chem, elastic_enabled.
void refk_phi_rhs(const double *phi, const double *eta, const double *xB, double *rhs, int n, const double *d,
                  const int *i, const float *sig, const float *eps, const double *Sp, const double *e00) {
    REF_LAUNCH(n, compute_phi_rhs_kernel(
        phi, eta, xB, rhs, n, 1, 1, d[0], d[1], d[2], d[3], d[4], d[5], d[6], d[7], d[8],
        sig, sig + n, sig + 2 * n, sig + 5 * n, sig + 4 * n, sig + 3 * n,
        eps, eps + n, eps + 2 * n, eps + 5 * n, eps + 4 * n, eps + 3 * n,
        Sp[0], Sp[1], Sp[2], Sp[3], Sp[4], Sp[5], Sp[6], Sp[7], Sp[8], Sp[9], Sp[10], Sp[11], Sp[12], Sp[13],
        Sp[14], Sp[15], Sp[16], Sp[17], Sp[18], Sp[19], Sp[20],
        e00[0], e00[1], e00[2], e00[3], e00[4], e00[5], d[9], i[0], i[1], i[2], d[10], d[11], d[12], i[3], n,
        i[4], (double *)nullptr));
}

// compute_eta_rhs_kernel (non-raw-drive branch) over n cells.  d: T_K,
// mu_reference_scale, Vm_alpha_0, dVm_alpha_dxB, gp_xB_fixed, gp_delta_g0,
// gp_W_eta, eps_iso_over_vB, gp_eps_iso, gp_elastic_derivative_scale.
// i: gp_elastic_enabled, gp_elastic_active_eta.
void refk_eta_rhs(const double *eta, const double *phi, const double *xB, double *rhs, int n, const double *d,
                  const int *i, const float *sig) {
    REF_LAUNCH(n, compute_eta_rhs_kernel(
        eta, phi, xB, sig, sig + n, sig + 2 * n, sig + 5 * n, sig + 4 * n, sig + 3 * n, rhs,
        d[0], d[1], d[2], d[3], d[4], d[5], 0, 0, 0.0, 0.0, 0.0, d[6], d[7], i[0], i[1], d[8], d[9], n,
        (double *)nullptr));
}

// compute_mu_x_kernel (gp = 0) or compute_mu_C_gp_kernel (gp = 1) over n
// cells; xB out as the kernels write it.  d: T_K, mu_reference_scale, v_A,
// v_B, mu0_compound, Vm_compound, Vm_alpha_0, dVm_alpha_dxB, Y_clip, xB_eps,
// eps_iso_over_vB.  sig: 6 n floats (the first three are read).
void refk_mu(int gp, const double *Y, const double *phi, double *xB, double *mu, int n, const double *d,
             const float *sig, int elastic) {
    if (gp)
        REF_LAUNCH(n, compute_mu_C_gp_kernel(Y, xB, mu, d[0], d[1], d[6], d[7], d[8], d[9], sig, sig + n,
                                             sig + 2 * n, d[10], n, elastic));
    else
        REF_LAUNCH(n, compute_mu_x_kernel(Y, phi, xB, mu, d[0], d[1], d[2], d[3], d[4], d[5], d[6], d[7], d[8],
                                          d[9], sig, sig + n, sig + 2 * n, d[10], n, elastic));
}

// compute_Y_rhs_kernel (zm = 0) or compute_Y_rhs_sm_tangent_n_kernel (zm = 1)
// over n cells.  d: dt, v_B, mean_DY, term_h_scale.  i: previous time
// level, gamma term disabled.
void refk_y_rhs(int zm, const double *divJ, const double *phi_new, const double *phi_old, const double *lapY,
                const double *Y, const double *dYdt, double *rhs, int n, const double *d, const int *i) {
    if (zm)
        REF_LAUNCH(n, compute_Y_rhs_sm_tangent_n_kernel(divJ, phi_old, phi_new, lapY, Y, dYdt, rhs, d[0], d[1],
                                                        d[2], n, (double *)nullptr));
    else
        REF_LAUNCH(n, compute_Y_rhs_kernel(divJ, phi_new, phi_old, lapY, Y, dYdt, rhs, d[0], d[1], d[2], n, i[0],
                                           i[1], d[3], (double *)nullptr));
}

// compute_strain_with_perturbation_kernel over n cells: the strains
// (6 n floats, xx yy zz yz xz xy) to the polarization written the same way.
// S, Sp: the 21 entries each; e00: xx yy zz yz xz xy; E0 likewise.
// i: gp_mode_enabled, gp_elastic_enabled.  d: eps_iso_over_vB, gp_eps_iso.
void refk_polarization(const float *eps, const double *phi, const double *eta, const double *xB, float *out,
                       int n, const float *S, const float *Sp, const float *e00, const float *E0, const double *d,
                       const int *i) {
    REF_LAUNCH(n, compute_strain_with_perturbation_kernel(
        eps, eps + n, eps + 2 * n, eps + 5 * n, eps + 4 * n, eps + 3 * n, phi, eta, xB,
        out, out + n, out + 2 * n, out + 5 * n, out + 4 * n, out + 3 * n,
        S[0], S[1], S[2], S[3], S[4], S[5], S[6], S[7], S[8], S[9], S[10], S[11], S[12], S[13], S[14], S[15],
        S[16], S[17], S[18], S[19], S[20],
        Sp[0], Sp[1], Sp[2], Sp[3], Sp[4], Sp[5], Sp[6], Sp[7], Sp[8], Sp[9], Sp[10], Sp[11], Sp[12], Sp[13],
        Sp[14], Sp[15], Sp[16], Sp[17], Sp[18], Sp[19], Sp[20],
        e00[0], e00[1], e00[2], e00[3], e00[4], e00[5], d[0], i[0], i[1], d[1],
        E0[0], E0[1], E0[2], E0[3], E0[4], E0[5], n));
}

// compute_displacement_from_hij_green_kernel over the Nk points of an
// Nx x Ny x Nz grid: tau (6 Nk cufftComplex, xx yy zz yz xz xy) to u (3 Nk).
void refk_green(const cufftComplex *tau, cufftComplex *u, int Nx, int Ny, int Nz, const float *S, double dx,
                double dy, double dz) {
    const int NzC = Nz / 2 + 1, nk = Nx * Ny * NzC;
    REF_LAUNCH(nk, compute_displacement_from_hij_green_kernel(
        tau, tau + nk, tau + 2 * nk, tau + 5 * nk, tau + 4 * nk, tau + 3 * nk, u, u + nk, u + 2 * nk,
        S[0], S[1], S[2], S[3], S[4], S[5], S[6], S[7], S[8], S[9], S[10], S[11], S[12], S[13], S[14], S[15],
        S[16], S[17], S[18], S[19], S[20], Nx, Ny, Nz, NzC, dx, dy, dz, nk));
}

// two_phase_storage_exact_Y_update_kernel over n cells.  d: dt, v_B, Y_clip,
// Y_upper_cap, xB_eps, h_alpha_eps.
void refk_storage_exact(const double *divJ, const double *phi_new, const double *phi_old, const double *Y_old,
                        double *Y, double *xB, int n, const double *d) {
    REF_LAUNCH(n, two_phase_storage_exact_Y_update_kernel(divJ, phi_new, phi_old, Y_old, Y, xB, d[0], d[1], d[2],
                                                          d[3], d[4], d[5], (double *)nullptr, n));
}

// compute_flux_single_component_kernel (gp = 0) or the _gp_ variant over n
// cells.  d: D_alpha, D_compound, Vm_alpha_0, dVm_alpha_dxB, Vm_compound,
// T_K, mu_reference_scale, gp_M_GP, gp_M_beta.
void refk_flux(int gp, const double *g, const double *phi, const double *eta, const double *xB_prev, double *J,
               int n, const double *d) {
    if (gp)
        REF_LAUNCH(n, compute_flux_single_component_gp_kernel(g, phi, eta, xB_prev, J, d[0], d[7], d[8], d[2], d[3],
                                                              d[4], d[5], d[6], n));
    else
        REF_LAUNCH(n, compute_flux_single_component_kernel(g, phi, xB_prev, J, d[0], d[1], d[2], d[3], d[4], d[5],
                                                           d[6], n));
}

// compute_xB_storage_rhs_kernel over n cells (lap normalised).  d: dt, v_B,
// mean_Dx, h_alpha_eps (the matrix storage floor).
void refk_xsplit_source(const double *divJ, const double *phi_new, const double *phi_old, const double *lap,
                        const double *xB_old, double *rhs, int n, const double *d) {
    REF_LAUNCH(n, compute_xB_storage_rhs_kernel(divJ, phi_new, phi_old, lap, xB_old, rhs, d[0], d[1], d[2], d[3],
                                                n));
}

// xB_normalize_clamp_and_logit_kernel over n cells (x normalised: invN 1);
// xB holds the previous composition on entry.  d: xB_eps, Y_clip,
// Y_upper_cap.
void refk_xsplit_final(const double *x, double *xB, double *Y, int n, const double *d) {
    REF_LAUNCH(n, xB_normalize_clamp_and_logit_kernel(const_cast<double *>(x), xB, Y, 1.0, d[0], d[1], d[2], n));
}

// q_transport_projection_split kernels over n cells; stats: PF_Q_STATS_COUNT
// doubles (the caller zeroes them and sets PF_Q_MIN_ALPHA to 1).
int refk_q_stats_layout(int *infeasible, int *violations) {
    *infeasible = PF_Q_INFEASIBLE_PHASE_COUNT;
    *violations = PF_Q_TRANSPORT_BOUND_VIOLATION_COUNT;
    return PF_Q_STATS_COUNT;
}
// apply_local_phase_storage_transfer_q_kernel (feasibility tolerance 1e-12)
void refk_q_phase(const double *phi_new, const double *phi_old, double *q, double vB, double *stats, int n) {
    REF_LAUNCH(n, apply_local_phase_storage_transfer_q_kernel(phi_new, phi_old, q, vB, 1.0e-12, stats, n));
}
// q_explicit_transport_and_reconstruct_kernel.  d: dt, xB_eps, Y_clip, Y_upper_cap
void refk_q_transport(double *q, const double *divJ, const double *phi, double *xB, double *Y, int n,
                      const double *d, double *stats) {
    REF_LAUNCH(n, q_explicit_transport_and_reconstruct_kernel(q, divJ, phi, xB, Y, d[0], d[1], d[2], d[3], 1.0e-12,
                                                              stats, n));
}
// q_normalize_validate_and_reconstruct_kernel in place, invN = 1.  d: xB_eps, Y_clip, Y_upper_cap
void refk_q_reconstruct(double *q, const double *phi, double *xB, double *Y, int n, const double *d,
                        double *stats) {
    REF_LAUNCH(n, q_normalize_validate_and_reconstruct_kernel(q, q, phi, xB, Y, 1.0, d[0], d[1], d[2], 1.0e-12,
                                                              stats, n));
}
// compute_flux_single_component_q_kernel.  d as refk_flux
void refk_flux_q(const double *g, const double *phi, const double *xB_prev, double *J, int n, const double *d) {
    REF_LAUNCH(n, compute_flux_single_component_q_kernel(g, phi, xB_prev, J, d[0], d[2], d[3], d[4], d[5], d[6], n));
}

// the conservative composition modes' kernels over an Nx x Ny x Nz grid;
// stats: PF_CONS_STATS_COUNT doubles, zeroed by the caller
int refk_cons_stats_layout(int *limited, int *constrained, int *violations, int *nonfinite) {
    *limited = PF_CONS_LIMITED_FACE_COUNT;
    *constrained = PF_CONS_PHASE_CONSTRAINT_COUNT;
    *violations = PF_CONS_BOUND_VIOLATION_COUNT;
    *nonfinite = PF_CONS_NONFINITE_COUNT;
    return PF_CONS_STATS_COUNT;
}
void refk_cons_init(const double *phi, const double *xB, double *storage, double vB, int ctot, int n) {
    REF_LAUNCH(n, initialize_conservative_storage_kernel(phi, xB, storage, vB, ctot, n));
}
// d: T_K, v_B, beta_support_eps, xB_eps, Y_clip
void refk_cons_context(const double *storage, const double *phi, double *xB, double *Y, int ctot, int n,
                       const double *d, double *stats) {
    REF_LAUNCH(n, reconstruct_conservative_context_kernel(storage, phi, xB, Y, d[0], d[1], ctot, d[2], d[3], d[4],
                                                          stats, n));
}
// d: spacing, dt, D_alpha, Vm_alpha_0, dVm_alpha_dxB, Vm_compound, T_K, mu_reference_scale, v_B, bound_tol
void refk_cons_sweep(double *storage, const double *mu, const double *phi, const double *xB, int Nx, int Ny, int Nz,
                     int axis, int parity, int ctot, int be, const double *d, double *stats) {
    const int n = Nx * Ny * Nz;
    REF_LAUNCH(n, pairwise_conservative_face_sweep_kernel(storage, mu, phi, xB, Nx, Ny, Nz, axis, parity, d[0], d[1],
                                                          d[2], d[3], d[4], d[5], d[6], d[7], d[8], ctot, be, d[9],
                                                          stats, n));
}
// d: T_K, v_B, beta_support_eps, xB_eps, Y_clip, bound_tol
void refk_cons_constrain(double *phi_new, const double *phi_old, double *storage, double *xB, double *Y, int ctot,
                         int n, const double *d, double *stats) {
    REF_LAUNCH(n, constrain_phase_and_reconstruct_conservative_kernel(phi_new, phi_old, storage, xB, Y, d[0], d[1],
                                                                      ctot, d[2], d[3], d[4], d[5], stats, n));
}

// dealias_23_kernel on a half spectrum of an Nx x Ny x Nz grid, in place
// GP storage coupling.  compute_Y_rhs_gp_kernel (conservative = 0) or
// compute_Y_rhs_gp_conservative_kernel (1) over n cells.  d: dt, gp_xB_fixed,
// mean_DY, gp_h_alpha_eps; i: use_previous_time_level, disable_gamma_term.
void refk_gp_y_rhs(int conservative, const double *divJ, const double *phi, const double *phi_prev,
                   const double *eta, const double *eta_prev, const double *lapY, const double *Y,
                   const double *dYdt, double *rhs, int n, const double *d, const int *i) {
    if (conservative)
        REF_LAUNCH(n, compute_Y_rhs_gp_conservative_kernel(divJ, phi, phi_prev, eta, eta_prev, lapY, Y, dYdt, rhs,
                                                           d[0], d[1], d[2], n, i[0], i[1], nullptr));
    else
        REF_LAUNCH(n, compute_Y_rhs_gp_kernel(divJ, phi, phi_prev, eta, eta_prev, lapY, Y, dYdt, rhs, d[0], d[1],
                                              d[2], d[3], n, i[0], i[1], nullptr));
}

// gp_storage_exact_Y_update_kernel (picard = 0) or iters sweeps of
// gp_picard_storage_Y_update_kernel (Y holds the guess on entry).  d: dt,
// gp_xB_fixed, Y_clip, Y_upper_cap, xB_eps, gp_h_alpha_eps.
void refk_gp_storage(int picard, int iters, const double *divJ, const double *phi_new, const double *phi_old,
                     const double *eta_new, const double *eta_old, const double *Y_old, double *Y, double *xB,
                     int n, const double *d) {
    if (!picard) {
        REF_LAUNCH(n, gp_storage_exact_Y_update_kernel(divJ, phi_new, phi_old, eta_new, eta_old, Y_old, Y, xB,
                                                       d[0], d[1], d[2], d[3], d[4], d[5], 0, nullptr, n));
        return;
    }
    for (int it = 0; it < iters; ++it)
        REF_LAUNCH(n, gp_picard_storage_Y_update_kernel(divJ, phi_new, phi_old, eta_new, eta_old, Y_old, Y, xB,
                                                        d[0], d[1], d[2], d[3], d[4], nullptr, n));
}

// gp_eta_feasibility_and_limiter_kernel over n cells (eta in place); the
// limited-cell count is returned.  d: dt, gp_xB_fixed, xB_min, xB_max,
// gp_h_alpha_eps.
double refk_gp_eta_feasibility(double *eta, const double *eta_old, const double *phi_new, const double *phi_old,
                               const double *xB_old, const double *divJ, int limiter, int n, const double *d) {
    double stats[GP_ETA_FEAS_STATS_COUNT] = {0.0};
    REF_LAUNCH(n, gp_eta_feasibility_and_limiter_kernel(eta, eta_old, phi_new, phi_old, xB_old, divJ, d[0], d[1],
                                                        d[2], d[3], d[4], limiter, stats, n));
    return stats[GP_ETA_FEAS_LIMITER_COUNT];
}

// reduce_sum_DY_gp_kernel with one-thread blocks: the per-cell terms
// h_alpha D_alpha x (1 - x) in out
void refk_gp_dy_terms(const double *Y, const double *phi, const double *eta, double *out, double D_alpha, int n) {
    REF_LAUNCH(n, reduce_sum_DY_gp_kernel(Y, phi, eta, out, D_alpha, n));
}

// reduce_sum_xBtot_gp_kernel with one-thread blocks: the per-cell xBtot_gp
void refk_gp_xbtot_terms(const double *phi, const double *eta, const double *xB, double *out, double xgp, int n) {
    REF_LAUNCH(n, reduce_sum_xBtot_gp_kernel(phi, eta, xB, out, xgp, n));
}

void refk_dealias(cuDoubleComplex *k, int Nx, int Ny, int Nz, double dx, double dy, double dz) {
    const int NzC = Nz / 2 + 1, nk = Nx * Ny * NzC;
    REF_LAUNCH(nk, dealias_23_kernel(k, Nx, Ny, Nz, NzC, dx, dy, dz, nk));
}

}  // extern "C"
