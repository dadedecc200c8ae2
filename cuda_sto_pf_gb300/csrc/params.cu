// params.cu — host-side parameter defaults, derived thermodynamics, status
// strings.  No device code.
#include <math.h>
#include <stdarg.h>
#include <string.h>

#include "common.cuh"

// SGTE unary Gibbs energy GHSER(T) = a + bT + cT lnT + dT^2 + eT^3 + f/T + gT^-9,
// two temperature ranges per element (data of thermo_utils.h:280-302).
namespace {
struct Sgte { double Tmax, a, b, c, d, e, f, g; };
const Sgte kPb[2] = {{600.61, -7650.085, 101.700244, -24.5242231, -0.00365895, -2.4395e-7, 0.0, 0.0},
                     {1e300, -10531.095, 154.243182, -32.4913959, 0.00154613, 0.0, 0.0, 8.05448e25}};
const Sgte kAg[2] = {{1234.93, -7209.512, 118.202013, -23.8463314, -0.001790585, -3.98587e-7, -12011.0, 0.0},
                     {1e300, -15095.252, 190.266404, -33.472, 0.0, 0.0, 0.0, 1.411773e29}};
const Sgte kTe[2] = {{722.66, -10544.679, 183.372894, -35.6687, 0.01583435, -5.240417e-6, 155015.0, 0.0},
                     {1e300, 9160.595, -129.265373, 13.004, -0.0362361, 5.006367e-6, 0.0, -1.28681e30}};
double sgte(const Sgte *t, double T) {
    const Sgte &r = (T < t[0].Tmax) ? t[0] : t[1];
    double v = r.a + r.b * T + r.c * T * log(T);
    v += r.d * T * T;
    if (r.e != 0.0) v += r.e * pow(T, 3);
    if (r.f != 0.0) v += r.f / T;
    if (r.g != 0.0) v += r.g * pow(T, -9);
    return v;
}
double Lparam(double T) { return 41212.9 - 18.05 * T; }
double scale_guard(double s) { return (fabs(s) < 1e-30) ? ((s >= 0.0) ? 1e-30 : -1e-30) : s; }
}  // namespace

double pfgb_host_G_PbTe(double T) { return (-76063.2138 + 9.67716633 * T) + sgte(kPb, T) + sgte(kTe, T); }
double pfgb_host_G_Ag2Te(double T) {
    double g = (-10128.93 - 12.645115 * T) + (2.0 / 3.0) * sgte(kAg, T) + (1.0 / 3.0) * sgte(kTe, T);
    return 3.0 * g;
}

void pfgb_thermo_const(double T, double scale, int convex, ThermoConst *tc) {
    const double s = scale_guard(scale);
    const double GA = pfgb_host_G_PbTe(T), GB = pfgb_host_G_Ag2Te(T);
    const double RT = PFGB_RGAS * T, L = Lparam(T);
    tc->GA_s = GA / s;
    tc->GB_s = GB / s;
    tc->RT_s = RT / s;
    tc->L_s = L / s;
    tc->convex = convex ? 1 : 0;
    const double xc = PFGB_XC_CONVEX;
    // offsets (mu - G)/s and slopes at xc of the CALPHAD expressions
    tc->muA_c = (RT * log(1.0 - xc) + L * xc * xc) / s;
    tc->muB_c = (RT * log(xc) + L * (1.0 - xc) * (1.0 - xc)) / s;
    tc->dmuA_c = (-RT / (1.0 - xc) + 2.0 * L * xc) / s;
    tc->dmuB_c = (RT / xc - 2.0 * L * (1.0 - xc)) / s;
    tc->Kpen_s = 5000.0 / s;
    tc->ddmu_c = tc->dmuB_c - tc->dmuA_c;
}

namespace {
// solubility limit: Newton on RT ln x + L (1-x)^2 = 0 (solve_x_eq_device,
// thermo_utils.h:427-452)
double xB_eq(double T) {
    double L = Lparam(T), RT = PFGB_RGAS * T;
    double x = exp(-L / RT);
    if (x < 1e-9) x = 1e-9;
    if (x > 0.99) x = 0.5;
    for (int it = 0; it < 20; ++it) {
        double f = RT * log(x) + L * (1.0 - x) * (1.0 - x);
        double df = RT / x - 2.0 * L * (1.0 - x);
        double d = f / df;
        x -= d;
        if (x < 1e-10) x = 1e-10;
        if (x > 0.999) x = 0.999;
        if (fabs(d) < 1e-8) break;
    }
    return x;
}
}  // namespace

extern "C" {

size_t pfgb_params_size(void) { return sizeof(pfgb_params); }

// Defaults of params_default() (main_cuda.cu:15781-16439) for the fields on
// the hot path.  Physical parameters the reference marks "must come from the
// parameter file" (-1 sentinels) are left at -1.
void pfgb_params_default(pfgb_params *p) {
    memset(p, 0, sizeof(*p));
    p->Nx = p->Ny = p->Nz = 400;
    p->model_mode = PFGB_MODEL_TWO_PHASE;
    p->mode = PFGB_MODE_DYNAMICS;
    p->precision = PFGB_PREC_FP64;
    p->elastic_precision = PFGB_PREC_FP32;
    p->thermo_convex_extrapolation_enabled = 0;
    p->dx = p->dy = p->dz = -1.0;
    p->dt = 1.0e-2;
    p->temperature_C = -1.0;
    p->mu_reference_scale = -1.0;
    p->W = p->kappa_phi = p->L_phi = -1.0;
    p->D_alpha = p->D_compound = -1.0;
    p->v_A = p->v_B = -1.0;
    p->Vm_compound = p->Vm_alpha_0 = p->dVm_alpha_dxB = -1.0;
    p->Y_clip = 20.0;
    p->xB_eps = 1e-8;
    p->elastic_shift_dimless = -1.0;
    p->elastic_enabled = 1;
    p->elastic_warm_start_enabled = 1;
    p->elastic_residual_control_enabled = 1;
    p->elastic_iter_min = 2;
    p->elastic_iter_max = 32;
    p->elastic_fail_on_nonconvergence = 1;
    p->elastic_increment_form = 1;
    p->pf_y_update_mode = PFGB_Y_LAGGED_RHS;
    p->gp_h_alpha_eps = 1.0e-8;   // main_cuda.cu:16187
    p->pf_matrix_storage_floor = 0.1;                      // main_cuda.cu:16116
    p->pf_composition_mode = PFGB_COMPOSITION_LEGACY;      // main_cuda.cu:16108-16114
    p->pf_conservative_flux_strategy = PFGB_CONS_FLUX_PAIRWISE_LIMITED;
    p->pf_conservative_bound_tol = 1.0e-12;
    p->pf_conservative_mass_tol = 1.0e-10;
    p->pf_conservative_beta_support_eps = 1.0e-10;
    p->pf_conservative_max_subcycles = 64;
    p->pf_composition_stabilizer_Dalpha_multiplier = 10.0; // main_cuda.cu:16117
    p->gp_barrier_only_mode = 1;                           // main_cuda.cu:15823
    p->enable_legacy_gp_storage_coupling = 0;              // main_cuda.cu:15824
    p->gp_y_update_mode = PFGB_GP_Y_OLD_RHS;               // main_cuda.cu:16188-16190
    p->gp_eta_mass_limiter = PFGB_GP_ETA_LIMITER_OFF;
    p->gp_y_picard_iters = 3;
    p->elastic_residual_tolerance = 1.0e-6;
    p->elastic_residual_absolute_floor = 1.0e-30;
    p->eps_iso_over_vB = -1.0;
    for (int i = 0; i < 6; ++i) { p->eps00[i] = -1.0; p->E0[i] = 0.0; }
    for (int i = 0; i < 21; ++i) { p->S[i] = -1.0; p->S_p[i] = -1.0; }
    p->enable_Y_rhs_previous_time_level = 0;
    p->disable_Y_rhs_gamma_term = 0;
    p->Y_rhs_term_h_scale = 1.0;
    p->zero_mode_enabled = 0;
    p->zero_mode_max_iterations = 24;          // main_cuda.cu:22487-22488
    p->zero_mode_tolerance_relative = 1.0e-12;
    p->gp_xB_fixed = 0.3529411764705882;
    p->gp_delta_g0 = 0.0;
    p->gp_W_eta = p->gp_kappa_eta = p->gp_L_eta = 0.0;
    p->gp_M_GP = p->gp_M_beta = 0.0;
    p->gp_eps_iso = 0.0;
    p->gp_elastic_derivative_scale = 1.0;
    p->minimize_full_model = 0;
    p->minimize_post_projection_iters = 1;
    p->minimize_max_iter = 2000;
    p->minimize_convergence_steps = 10;
    p->minimize_dt = 1.0e-2;
    p->minimize_V0 = 0.0;
    p->eta_lambda_vol = 0.2;
    p->minimize_xB_max_safe = 0.07;
    p->minimize_min_pseudo_time = 0.0;
    p->ic_23d_xB_out = 0.03;        // params_default, main_cuda.cu:16215
    p->ic_phi_seed_radius = 10.0;   // main_cuda.cu:16221
    p->ic_phi_num_seeds = 1;
    // seeded initialisation (main_cuda.cu:16226-16238, 15791)
    p->init_shape_mode = -1;
    p->init_use_rotation = 0;
    p->init_axis_ratio_rx = p->init_axis_ratio_ry = p->init_axis_ratio_rz = 1.0;
    p->seed = 12345;
    p->minimize_rms_dphi_threshold = 1.0e-6;
    p->minimize_rms_dY_threshold = 5.0e-5;
    p->minimize_energy_diff_rel_threshold = 1.0e-9;
    p->minimize_rms_res_threshold = 1.0e-4;
    p->minimize_vol_err_rel_threshold = 1.0e-4;
}

// pfparams_refresh_thermo (main_cuda.cu:15603-15613)
pfgb_status pfgb_params_finalize(pfgb_params *p) {
    if (!p) return PFGB_ERR_INVALID;
    double T = p->temperature_C + 273.15;
    if (T < 1.0) T = 1.0;
    p->temperature_K = T;
    const double xeq = xB_eq(T);
    p->xB_eq_matrix = xeq;
    ThermoConst tc;
    pfgb_thermo_const(T, p->mu_reference_scale, p->thermo_convex_extrapolation_enabled, &tc);
    double muA, muB;
    thermo_mu<double>(tc, xeq, muA, muB);
    double vs = p->v_A + p->v_B;
    if (fabs(vs) < 1e-30) vs = (vs >= 0.0) ? 1e-30 : -1e-30;
    p->mu0_compound = (p->v_A * muA + p->v_B * muB) / vs;
    return PFGB_OK;
}

const char *pfgb_status_string(pfgb_status s) {
    switch (s) {
        case PFGB_OK: return "ok";
        case PFGB_ERR_INVALID: return "invalid argument";
        case PFGB_ERR_CUDA: return "CUDA error";
        case PFGB_ERR_NOMEM: return "device out of memory";
        case PFGB_ERR_NONCONVERGED: return "elastic solver did not converge";
        case PFGB_ERR_ZERO_MODE: return "zero-mode mass solve rejected the step";
        case PFGB_ERR_NONFINITE: return "non-finite value";
        case PFGB_ERR_TIMEOUT: return "bounded device wait timed out";
        case PFGB_ERR_UNSUPPORTED: return "unsupported option";
    }
    return "unknown status";
}

// load_raw_init_fields clamping rules (main_cuda.cu:2904-2990)
pfgb_status pfgb_prepare_raw_fields(const pfgb_params *p, double xB_max_safe, double *phi,
                                    double *xB, double *eta, const double *dYdt, size_t n) {
    if (!p || !phi || !xB) return PFGB_ERR_INVALID;
    for (size_t i = 0; i < n; ++i) {
        const double e = eta ? eta[i] : 0.0, d = dYdt ? dYdt[i] : 0.0;
        if (!isfinite(phi[i]) || !isfinite(xB[i]) || !isfinite(e) || !isfinite(d))
            return PFGB_ERR_NONFINITE;
        phi[i] = clamp01(phi[i]);
        if (eta) eta[i] = clamp01(eta[i]);
        double x = clamp_eps(xB[i], p->xB_eps);
        if (isfinite(xB_max_safe) && x > xB_max_safe) x = xB_max_safe;
        xB[i] = x;
    }
    return PFGB_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// last-error storage (thread local: one context per thread)
// ---------------------------------------------------------------------------
static thread_local char g_err[512];

void pfgb_set_error(const char *what, cudaError_t e, const char *file, int line) {
    snprintf(g_err, sizeof(g_err), "%s failed: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
}
void pfgb_set_error_msg(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}
const char *pfgb_error_buffer(void) { return g_err; }
