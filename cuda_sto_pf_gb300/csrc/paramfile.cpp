// paramfile.cpp — `key=value` parameter files for pfgb_params.
//
// Same contract as the reference loader (load_pfparams_override_file,
// main_cuda.cu:22306-22360, apply_pfparams_override_key :21226+): '#'
// starts a comment, blank lines are skipped, `key=value` with surrounding
// whitespace trimmed, unknown keys are warned about and ignored, a value that
// does not parse completely as a number is an error, and after the file the
// required physical keys (validate_required_pfparams_presence, :1089-1146)
// must all have been seen, including the full eps*00, S_* and S_p_* sets.
#include <cctype>
#include <cerrno>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "pfgb.h"

namespace {

bool parse_double(const char *s, double *out) {
    if (!s || !*s) return false;
    errno = 0;
    char *end = nullptr;
    double v = strtod(s, &end);
    if (errno == ERANGE || end == s) return false;
    while (*end && isspace((unsigned char)*end)) ++end;
    if (*end) return false;
    *out = v;
    return true;
}

bool parse_int(const char *s, int *out) {
    if (!s || !*s) return false;
    errno = 0;
    char *end = nullptr;
    long v = strtol(s, &end, 10);
    if (errno == ERANGE || end == s || v < -2147483647L || v > 2147483647L) return false;
    while (*end && isspace((unsigned char)*end)) ++end;
    if (*end) return false;
    *out = (int)v;
    return true;
}

// Voigt suffix "11".."66" (a <= b) -> index into the 21-vector
int voigt21(const char *suf) {
    if (strlen(suf) != 2) return -1;
    int a = suf[0] - '1', b = suf[1] - '1';
    if (a < 0 || a > 5 || b < a || b > 5) return -1;
    static const int start[6] = {0, 6, 11, 15, 18, 20};
    return start[a] + (b - a);
}

const char *kEigen[6] = {"eps_xx00", "eps_yy00", "eps_zz00", "eps_yz00", "eps_xz00", "eps_xy00"};
const char *kE0[6] = {"E0_xx", "E0_yy", "E0_zz", "E0_yz", "E0_xz", "E0_xy"};

struct DKey { const char *name; size_t off; };
#define DK(n, f) {n, offsetof(pfgb_params, f)}
const DKey kDoubles[] = {
    DK("dt", dt), DK("dx", dx), DK("dy", dy), DK("dz", dz), DK("t_real_unit", t_real_unit),
    DK("temperature_C", temperature_C), DK("mu_reference_scale", mu_reference_scale),
    DK("W", W), DK("kappa_phi", kappa_phi), DK("L_phi", L_phi), DK("D_alpha", D_alpha),
    DK("D_compound", D_compound), DK("v_A", v_A), DK("v_B", v_B), DK("Vm_compound", Vm_compound),
    DK("Vm_alpha_0", Vm_alpha_0), DK("dVm_alpha_dxB", dVm_alpha_dxB), DK("Y_clip", Y_clip),
    DK("xB_eps", xB_eps), DK("elastic_shift_dimless", elastic_shift_dimless),
    DK("eps_iso_over_vB", eps_iso_over_vB), DK("elastic_residual_tolerance", elastic_residual_tolerance),
    DK("elastic_residual_absolute_floor", elastic_residual_absolute_floor),
    DK("Y_rhs_term_h_scale", Y_rhs_term_h_scale), DK("gp_xB_fixed", gp_xB_fixed),
    DK("gp_delta_g0", gp_delta_g0), DK("gp_W_eta_code", gp_W_eta), DK("gp_kappa_eta_code", gp_kappa_eta),
    DK("gp_L_eta_code", gp_L_eta), DK("gp_W_eta", gp_W_eta), DK("gp_kappa_eta", gp_kappa_eta),
    DK("gp_L_eta", gp_L_eta), DK("gp_M_GP", gp_M_GP), DK("gp_M_beta", gp_M_beta),
    DK("gp_eps_iso", gp_eps_iso), DK("gp_elastic_derivative_scale", gp_elastic_derivative_scale),
    DK("minimize_dt", minimize_dt), DK("minimize_V0", minimize_V0), DK("eta_lambda_vol", eta_lambda_vol),
    DK("minimize_xB_max_safe", minimize_xB_max_safe),
    DK("minimize_rms_dphi_threshold", minimize_rms_dphi_threshold),
    DK("minimize_rms_dY_threshold", minimize_rms_dY_threshold),
    DK("minimize_energy_diff_rel_threshold", minimize_energy_diff_rel_threshold),
    DK("minimize_rms_res_threshold", minimize_rms_res_threshold),
    DK("minimize_vol_err_rel_threshold", minimize_vol_err_rel_threshold),
    DK("ic_vf_init_phi", ic_vf_init_phi), DK("ic_vf_target_phi", ic_vf_target_phi),
    DK("ic_phi_iface_w", ic_phi_iface_w), DK("gamma_Jm2", gamma_Jm2), DK("lambda_sm_m", lambda_sm_m),
    DK("Vm_alpha_0_phys_m3mol", Vm_alpha_0_phys_m3mol),
    DK("ic_23d_xB_out", ic_23d_xB_out), DK("xB_alpha_initial", ic_23d_xB_out),
    DK("ic_phi_seed_radius", ic_phi_seed_radius), DK("minimize_min_pseudo_time", minimize_min_pseudo_time),
    DK("init_axis_ratio_rx", init_axis_ratio_rx), DK("init_axis_ratio_ry", init_axis_ratio_ry),
    DK("init_axis_ratio_rz", init_axis_ratio_rz), DK("init_tilt_theta_deg", init_tilt_theta_deg),
    DK("init_tilt_phi_deg", init_tilt_phi_deg), DK("init_center_shift_x", init_center_shift_x),
    DK("init_center_shift_y", init_center_shift_y), DK("init_center_shift_z", init_center_shift_z),
    DK("init_phi_noise_amp", init_phi_noise_amp), DK("gp_h_alpha_eps", gp_h_alpha_eps),
    DK("pf_matrix_storage_floor", pf_matrix_storage_floor),
    DK("pf_conservative_bound_tol", pf_conservative_bound_tol),
    DK("pf_conservative_mass_tol", pf_conservative_mass_tol),
    DK("pf_conservative_beta_support_eps", pf_conservative_beta_support_eps),
    DK("pf_composition_stabilizer_Dalpha_multiplier", pf_composition_stabilizer_Dalpha_multiplier),
};
const DKey kInts[] = {
    DK("pf_params_schema_version", pf_params_schema_version),
    DK("thermo_convex_extrapolation_enabled", thermo_convex_extrapolation_enabled),
    DK("elastic_enabled", elastic_enabled), DK("elastic_warm_start_enabled", elastic_warm_start_enabled),
    DK("elastic_residual_control_enabled", elastic_residual_control_enabled),
    DK("elastic_iter_min", elastic_iter_min), DK("elastic_iter_max", elastic_iter_max),
    DK("elastic_fail_on_nonconvergence", elastic_fail_on_nonconvergence),
    DK("elastic_increment_form", elastic_increment_form),
    DK("elastic_warm_start_extrapolate", elastic_warm_start_extrapolate),
    DK("elastic_warm_start_source", elastic_warm_start_source),
    DK("elastic_chebyshev", elastic_chebyshev), DK("fft_tensor_cores", fft_tensor_cores),
    DK("fft_autotune", fft_autotune),
    DK("zero_mode_fp64_cells", zero_mode_fp64_cells),
    DK("pf_conservative_max_subcycles", pf_conservative_max_subcycles),
    DK("gp_y_picard_iters", gp_y_picard_iters), DK("gp_limiter_flux_from_xn", gp_limiter_flux_from_xn),
    DK("y_update_mass_projection_enabled", y_update_mass_projection_enabled),
    DK("enable_Y_rhs_previous_time_level", enable_Y_rhs_previous_time_level),
    DK("disable_Y_rhs_gamma_term", disable_Y_rhs_gamma_term),
    DK("gp_elastic_enabled", gp_elastic_enabled), DK("gp_elastic_active_eta", gp_elastic_active_eta),
    DK("gp_elastic_active_phi", gp_elastic_active_phi),
    DK("minimize_full_model", minimize_full_model),
    DK("minimize_post_projection_iters", minimize_post_projection_iters),
    DK("minimize_max_iter", minimize_max_iter), DK("minimize_convergence_steps", minimize_convergence_steps),
    DK("ic_phi_num_seeds", ic_phi_num_seeds),
    DK("init_shape_mode", init_shape_mode), DK("init_use_rotation", init_use_rotation),
};
#undef DK

// keys of the reference schema that do not drive this path (GP/event
// engines, converter provenance): accepted without a warning
// reference keys whose other values select paths this library does not
// build (pf_params.h; defaults at main_cuda.cu:15829, 15883, 16080, 16108,
// 16137, 16424): any other value is refused, not ignored
struct Selector { const char *key, *allowed; };
const Selector kSelectors[] = {
    {"enable_Y_rhs_picard", "0"},              {"enable_gp_assisted_beta_nucleation", "0"},
    {"gp_nuc_enabled", "0"},                   {"diagnostic_rsmd_enabled", "0"},
};

const char *kKnownUnused[] = {
    "gp_W_eta_phys", "gp_kappa_eta_phys", "gp_L_eta_phys", "gp_gamma_alpha_gp", "gp_l_eta_nm",
    "gp_D_ratio", "gp_reaction_nu_A", "gp_reaction_nu_B", "gp_xB_eq_alpha_for_eta",
    "gp_M_eta_ratio_to_crit", "gp_M_eta_phys", "gp_delta_g_stab",
};

enum { R_DT, R_DX, R_DY, R_DZ, R_TRU, R_TC, R_MUS, R_W, R_KAP, R_LPHI, R_DA, R_DC, R_VA, R_VB, R_VMC,
       R_VM0, R_DVM, R_ICI, R_ICT, R_ICW, R_GAM, R_LAM, R_VMP, R_SHIFT, R_EIV, R_SCHEMA, R_COUNT };
const char *kRequired[R_COUNT] = {
    "dt", "dx", "dy", "dz", "t_real_unit", "temperature_C", "mu_reference_scale", "W", "kappa_phi",
    "L_phi", "D_alpha", "D_compound", "v_A", "v_B", "Vm_compound", "Vm_alpha_0", "dVm_alpha_dxB",
    "ic_vf_init_phi", "ic_vf_target_phi", "ic_phi_iface_w", "gamma_Jm2", "lambda_sm_m",
    "Vm_alpha_0_phys_m3mol", "elastic_shift_dimless", "eps_iso_over_vB", "pf_params_schema_version"};

struct Presence { unsigned req = 0, eig = 0; unsigned s = 0, sp = 0; };

void mark(Presence &pr, const char *key) {
    for (int i = 0; i < R_COUNT; ++i)
        if (!strcmp(key, kRequired[i])) pr.req |= 1u << i;
    for (int i = 0; i < 6; ++i)
        if (!strcmp(key, kEigen[i])) pr.eig |= 1u << i;
    if (!strncmp(key, "S_p_", 4)) { int v = voigt21(key + 4); if (v >= 0) pr.sp |= 1u << v; }
    else if (!strncmp(key, "S_", 2)) { int v = voigt21(key + 2); if (v >= 0) pr.s |= 1u << v; }
}

void trim(std::string &s) {
    size_t a = 0, b = s.size();
    while (a < b && isspace((unsigned char)s[a])) ++a;
    while (b > a && isspace((unsigned char)s[b - 1])) --b;
    s = s.substr(a, b - a);
}

void seterr(char *buf, size_t n, const char *fmt, ...) {
    if (!buf || !n) return;
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, n, fmt, ap);
    va_end(ap);
}

}  // namespace

extern "C" pfgb_status pfgb_params_set(pfgb_params *p, const char *key, const char *value) {
    if (!p || !key || !value) return PFGB_ERR_INVALID;
    for (const auto &k : kDoubles)
        if (!strcmp(key, k.name)) {
            double v;
            if (!parse_double(value, &v)) return PFGB_ERR_INVALID;
            *(double *)((char *)p + k.off) = v;
            return PFGB_OK;
        }
    for (const auto &k : kInts)
        if (!strcmp(key, k.name)) {
            int v;
            if (!parse_int(value, &v)) return PFGB_ERR_INVALID;
            *(int32_t *)((char *)p + k.off) = v;
            return PFGB_OK;
        }
    for (int i = 0; i < 6; ++i) {
        if (!strcmp(key, kEigen[i])) return parse_double(value, &p->eps00[i]) ? PFGB_OK : PFGB_ERR_INVALID;
        if (!strcmp(key, kE0[i])) return parse_double(value, &p->E0[i]) ? PFGB_OK : PFGB_ERR_INVALID;
    }
    if (!strncmp(key, "S_p_", 4)) {
        int v = voigt21(key + 4);
        if (v >= 0) return parse_double(value, &p->S_p[v]) ? PFGB_OK : PFGB_ERR_INVALID;
    } else if (!strncmp(key, "S_", 2)) {
        int v = voigt21(key + 2);
        if (v >= 0) return parse_double(value, &p->S[v]) ? PFGB_OK : PFGB_ERR_INVALID;
    }
    if (!strcmp(key, "seed") || !strcmp(key, "init_phi_noise_seed")) {   // unsigned long (TRY_SET_ULONG)
        char *e = nullptr;
        errno = 0;
        const unsigned long long v = strtoull(value, &e, 10);
        if (e == value || *e != '\0' || errno != 0 || value[0] == '-') return PFGB_ERR_INVALID;
        (!strcmp(key, "seed") ? p->seed : p->init_phi_noise_seed) = (uint64_t)v;
        return PFGB_OK;
    }
    for (const Selector &sel : kSelectors)
        if (!strcmp(key, sel.key)) return strcmp(value, sel.allowed) ? PFGB_ERR_INVALID : PFGB_OK;
    if (!strcmp(key, "gp_barrier_only_mode") || !strcmp(key, "enable_legacy_gp_storage_coupling")) {
        char *e = nullptr;
        const long v = strtol(value, &e, 10);
        if (e == value || *e != '\0') return PFGB_ERR_INVALID;
        (!strcmp(key, "gp_barrier_only_mode") ? p->gp_barrier_only_mode : p->enable_legacy_gp_storage_coupling) =
            (int32_t)v;
        return PFGB_OK;
    }
    if (!strcmp(key, "pf_y_update_mode")) {   // pf_params.h:345, checked fatally at main_cuda.cu:1688-1696
        if (!strcmp(value, "lagged_rhs")) { p->pf_y_update_mode = PFGB_Y_LAGGED_RHS; return PFGB_OK; }
        if (!strcmp(value, "storage_exact")) { p->pf_y_update_mode = PFGB_Y_STORAGE_EXACT; return PFGB_OK; }
        if (!strcmp(value, "x_transport_projection_split")) {
            p->pf_y_update_mode = PFGB_Y_X_TRANSPORT_SPLIT;
            return PFGB_OK;
        }
        if (!strcmp(value, "q_transport_projection_split")) {
            p->pf_y_update_mode = PFGB_Y_Q_TRANSPORT_SPLIT;
            return PFGB_OK;
        }
        return PFGB_ERR_INVALID;
    }
    if (!strcmp(key, "gp_y_update_mode")) {   // main_cuda.cu:22254-22263
        if (!strcmp(value, "old_rhs")) { p->gp_y_update_mode = PFGB_GP_Y_OLD_RHS; return PFGB_OK; }
        if (!strcmp(value, "conservative_y_rhs")) { p->gp_y_update_mode = PFGB_GP_Y_CONSERVATIVE_RHS; return PFGB_OK; }
        if (!strcmp(value, "picard_storage")) { p->gp_y_update_mode = PFGB_GP_Y_PICARD_STORAGE; return PFGB_OK; }
        if (!strcmp(value, "storage_exact")) { p->gp_y_update_mode = PFGB_GP_Y_STORAGE_EXACT; return PFGB_OK; }
        return PFGB_ERR_INVALID;
    }
    if (!strcmp(key, "gp_eta_mass_limiter")) {   // main_cuda.cu:22244-22252 (off or local_clip)
        if (!strcmp(value, "off")) { p->gp_eta_mass_limiter = PFGB_GP_ETA_LIMITER_OFF; return PFGB_OK; }
        if (!strcmp(value, "local_clip")) { p->gp_eta_mass_limiter = PFGB_GP_ETA_LIMITER_LOCAL_CLIP; return PFGB_OK; }
        return PFGB_ERR_INVALID;
    }
    if (!strcmp(key, "pf_composition_mode")) {   // pf_params.h:349, checked at main_cuda.cu:1697-1703
        if (!strcmp(value, "legacy")) { p->pf_composition_mode = PFGB_COMPOSITION_LEGACY; return PFGB_OK; }
        if (!strcmp(value, "ctot_conservative_split")) { p->pf_composition_mode = PFGB_COMPOSITION_CTOT; return PFGB_OK; }
        if (!strcmp(value, "qalpha_conservative_local_transaction")) {
            p->pf_composition_mode = PFGB_COMPOSITION_QALPHA;
            return PFGB_OK;
        }
        return PFGB_ERR_INVALID;
    }
    if (!strcmp(key, "pf_conservative_flux_strategy")) {   // pf_params.h:350, main_cuda.cu:1705-1710
        if (!strcmp(value, "pairwise_limited")) {
            p->pf_conservative_flux_strategy = PFGB_CONS_FLUX_PAIRWISE_LIMITED;
            return PFGB_OK;
        }
        if (!strcmp(value, "pairwise_backward_euler")) {
            p->pf_conservative_flux_strategy = PFGB_CONS_FLUX_BACKWARD_EULER;
            return PFGB_OK;
        }
        return PFGB_ERR_INVALID;
    }
    if (!strcmp(key, "model_mode")) {
        if (!strcmp(value, "two_phase")) { p->model_mode = PFGB_MODEL_TWO_PHASE; return PFGB_OK; }
        if (!strcmp(value, "gp_zone")) { p->model_mode = PFGB_MODEL_GP_ZONE; return PFGB_OK; }
        return PFGB_ERR_INVALID;
    }
    for (const char *k : kKnownUnused)
        if (!strcmp(key, k)) {
            double v;
            return parse_double(value, &v) ? PFGB_OK : PFGB_ERR_INVALID;
        }
    return PFGB_ERR_UNSUPPORTED;
}

extern "C" pfgb_status pfgb_params_load_file(pfgb_params *p, const char *path, char *errbuf, size_t errlen) {
    if (!p || !path || !*path) {
        seterr(errbuf, errlen, "no parameter file given");
        return PFGB_ERR_INVALID;
    }
    FILE *fp = fopen(path, "r");
    if (!fp) {
        seterr(errbuf, errlen, "could not open pf-param file: %s", path);
        return PFGB_ERR_INVALID;
    }
    char line[4096];
    int line_no = 0;
    Presence pr;
    while (fgets(line, sizeof(line), fp)) {
        ++line_no;
        char *hash = strchr(line, '#');
        if (hash) *hash = '\0';
        std::string s(line);
        trim(s);
        if (s.empty()) continue;
        size_t eq = s.find('=');
        if (eq == std::string::npos) {
            seterr(errbuf, errlen, "%s:%d expected key=value format", path, line_no);
            fclose(fp);
            return PFGB_ERR_INVALID;
        }
        std::string key = s.substr(0, eq), val = s.substr(eq + 1);
        trim(key);
        trim(val);
        pfgb_status st = pfgb_params_set(p, key.c_str(), val.c_str());
        if (st == PFGB_ERR_INVALID) {
            bool selector = false;
            for (const Selector &sel : kSelectors) selector = selector || key == sel.key;
            if (selector)
                seterr(errbuf, errlen, "%s:%d %s=%s selects a path that is not built", path, line_no, key.c_str(),
                       val.c_str());
            else
                seterr(errbuf, errlen, "%s:%d invalid value for %s: %s", path, line_no, key.c_str(), val.c_str());
            fclose(fp);
            return PFGB_ERR_INVALID;
        }
        if (st == PFGB_ERR_UNSUPPORTED) {
            fprintf(stderr, "[warn] %s:%d unknown key ignored: %s\n", path, line_no, key.c_str());
            continue;
        }
        mark(pr, key.c_str());
    }
    fclose(fp);
    std::string missing;
    for (int i = 0; i < R_COUNT; ++i)
        if (!(pr.req & (1u << i))) { missing += missing.empty() ? "" : ","; missing += kRequired[i]; }
    if (pr.eig != 0x3fu) { missing += missing.empty() ? "" : ","; missing += "eps_xx00..eps_xy00"; }
    if (pr.s != 0x1fffffu) { missing += missing.empty() ? "" : ","; missing += "S_*"; }
    if (pr.sp != 0x1fffffu) { missing += missing.empty() ? "" : ","; missing += "S_p_*"; }
    if (!missing.empty()) {
        seterr(errbuf, errlen, "%s is missing required parameters: %s", path, missing.c_str());
        return PFGB_ERR_INVALID;
    }
    return PFGB_OK;
}
