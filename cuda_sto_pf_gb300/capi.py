"""ctypes binding of the pfgb C ABI (include/pfgb.h).

This is the Python host side above the C ABI: the same entry points a C/C++
caller links against.  There is no fallback: if libpfgb.so (built in-tree by
cuda_sto_pf_gb300.build) cannot be loaded, every call raises.
"""
from __future__ import annotations

import ctypes
import os
from ctypes import (POINTER, Structure, c_char_p, c_double, c_int, c_int32, c_size_t, c_void_p)

from . import build as _build

c_double_p = POINTER(c_double)
c_float_p = POINTER(ctypes.c_float)

PREC_FP64, PREC_FP32 = 0, 1
MODEL_TWO_PHASE, MODEL_GP_ZONE = 0, 1
MODE_DYNAMICS, MODE_MINIMIZE = 0, 1
Y_LAGGED_RHS, Y_STORAGE_EXACT, Y_X_TRANSPORT_SPLIT, Y_Q_TRANSPORT_SPLIT = 0, 1, 2, 3
COMPOSITION_LEGACY, COMPOSITION_CTOT, COMPOSITION_QALPHA = 0, 1, 2
CONS_FLUX_PAIRWISE_LIMITED, CONS_FLUX_BACKWARD_EULER = 0, 1
GP_Y_OLD_RHS, GP_Y_PICARD_STORAGE, GP_Y_STORAGE_EXACT, GP_Y_CONSERVATIVE_RHS = 0, 1, 2, 3
GP_ETA_LIMITER_OFF, GP_ETA_LIMITER_LOCAL_CLIP = 0, 1

STATUS = {0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "device out of memory",
          4: "elastic solver did not converge", 5: "zero-mode mass solve rejected the step",
          6: "non-finite value", 7: "bounded device wait timed out", 8: "unsupported option",
          9: "model file read/write failed"}

FNO_WIDTH, FNO_HIDDEN, FNO_IN, FNO_OUT = 32, 64, 8, 3
# elastic_warm_start_source
WARM_PREVIOUS, WARM_MODEL_COLD_STARTS, WARM_MODEL_EVERY_STEP, WARM_NONE = 0, 1, 2, 3


class Params(Structure):
    """Mirror of pfgb_params (field order and types must match pfgb.h)."""
    _fields_ = [
        ("Nx", c_int32), ("Ny", c_int32), ("Nz", c_int32),
        ("model_mode", c_int32), ("mode", c_int32), ("precision", c_int32),
        ("elastic_precision", c_int32), ("thermo_convex_extrapolation_enabled", c_int32),
        ("dx", c_double), ("dy", c_double), ("dz", c_double), ("dt", c_double),
        ("temperature_C", c_double), ("mu_reference_scale", c_double),
        ("W", c_double), ("kappa_phi", c_double), ("L_phi", c_double),
        ("D_alpha", c_double), ("D_compound", c_double),
        ("v_A", c_double), ("v_B", c_double),
        ("Vm_compound", c_double), ("Vm_alpha_0", c_double), ("dVm_alpha_dxB", c_double),
        ("Y_clip", c_double), ("xB_eps", c_double),
        ("elastic_shift_dimless", c_double),
        ("elastic_enabled", c_int32), ("elastic_warm_start_enabled", c_int32),
        ("elastic_residual_control_enabled", c_int32), ("elastic_iter_min", c_int32),
        ("elastic_iter_max", c_int32), ("elastic_fail_on_nonconvergence", c_int32),
        ("elastic_increment_form", c_int32), ("elastic_warm_start_extrapolate", c_int32),
        ("elastic_chebyshev", c_int32), ("fft_tensor_cores", c_int32), ("fft_autotune", c_int32), ("pad_fft", c_int32),
        ("elastic_residual_tolerance", c_double), ("elastic_residual_absolute_floor", c_double),
        ("eps_iso_over_vB", c_double),
        ("eps00", c_double * 6), ("E0", c_double * 6),
        ("S", c_double * 21), ("S_p", c_double * 21),
        ("enable_Y_rhs_previous_time_level", c_int32), ("disable_Y_rhs_gamma_term", c_int32),
        ("Y_rhs_term_h_scale", c_double),
        ("pf_y_update_mode", c_int32), ("pad_y", c_int32), ("gp_h_alpha_eps", c_double),
        ("pf_matrix_storage_floor", c_double), ("pf_composition_stabilizer_Dalpha_multiplier", c_double),
        ("gp_barrier_only_mode", c_int32), ("enable_legacy_gp_storage_coupling", c_int32),
        ("zero_mode_enabled", c_int32), ("zero_mode_max_iterations", c_int32),
        ("zero_mode_tolerance_relative", c_double),
        ("gp_elastic_enabled", c_int32), ("gp_elastic_active_eta", c_int32),
        ("gp_elastic_active_phi", c_int32), ("gp_pad0", c_int32),
        ("gp_xB_fixed", c_double), ("gp_delta_g0", c_double),
        ("gp_W_eta", c_double), ("gp_kappa_eta", c_double), ("gp_L_eta", c_double),
        ("gp_M_GP", c_double), ("gp_M_beta", c_double),
        ("gp_eps_iso", c_double), ("gp_elastic_derivative_scale", c_double),
        ("minimize_full_model", c_int32), ("minimize_post_projection_iters", c_int32),
        ("minimize_max_iter", c_int32), ("minimize_convergence_steps", c_int32),
        ("minimize_dt", c_double), ("minimize_V0", c_double), ("eta_lambda_vol", c_double),
        ("minimize_xB_max_safe", c_double),
        ("minimize_rms_dphi_threshold", c_double), ("minimize_rms_dY_threshold", c_double),
        ("minimize_energy_diff_rel_threshold", c_double), ("minimize_rms_res_threshold", c_double),
        ("minimize_vol_err_rel_threshold", c_double),
        ("pf_params_schema_version", c_int32), ("zero_mode_fp64_cells", c_int32),
        ("t_real_unit", c_double),
        ("ic_vf_init_phi", c_double), ("ic_vf_target_phi", c_double), ("ic_phi_iface_w", c_double),
        ("gamma_Jm2", c_double), ("lambda_sm_m", c_double), ("Vm_alpha_0_phys_m3mol", c_double),
        ("ic_23d_xB_out", c_double), ("ic_phi_seed_radius", c_double), ("minimize_min_pseudo_time", c_double),
        ("ic_phi_num_seeds", c_int32), ("elastic_warm_start_source", c_int32),
        ("init_shape_mode", c_int32), ("init_use_rotation", c_int32),
        ("init_axis_ratio_rx", c_double), ("init_axis_ratio_ry", c_double), ("init_axis_ratio_rz", c_double),
        ("init_tilt_theta_deg", c_double), ("init_tilt_phi_deg", c_double),
        ("init_center_shift_x", c_double), ("init_center_shift_y", c_double), ("init_center_shift_z", c_double),
        ("init_phi_noise_amp", c_double), ("init_phi_noise_seed", ctypes.c_uint64), ("seed", ctypes.c_uint64),
        ("pf_composition_mode", c_int32), ("pf_conservative_flux_strategy", c_int32),
        ("pf_conservative_bound_tol", c_double), ("pf_conservative_mass_tol", c_double),
        ("pf_conservative_beta_support_eps", c_double), ("pf_conservative_max_subcycles", c_int32),
        ("gp_y_update_mode", c_int32), ("gp_eta_mass_limiter", c_int32), ("gp_y_picard_iters", c_int32),
        ("gp_limiter_flux_from_xn", c_int32), ("y_update_mass_projection_enabled", c_int32),
        ("temperature_K", c_double), ("mu0_compound", c_double), ("xB_eq_matrix", c_double),
    ]


class StepStats(Structure):
    _fields_ = [
        ("step", c_int32), ("elastic_iterations", c_int32), ("elastic_converged", c_int32),
        ("elastic_warm_start_used", c_int32), ("elastic_relative_residual", c_double),
        ("elastic_iterations_total", c_int32), ("zero_mode_iterations", c_int32),
        ("zero_mode_newton_steps", c_int32), ("zero_mode_bisection_steps", c_int32),
        ("zero_mode_lambda", c_double), ("zero_mode_residual", c_double),
        ("zero_mode_target_mass", c_double), ("mean_DY", c_double),
        ("q_phase_rejected", c_int32), ("q_redistributed_cells", c_int32),
        ("cons_limited_faces", c_int32), ("cons_phase_constrained", c_int32),
        ("gp_eta_limited_cells", c_int32), ("pad_stats", c_int32),
    ]


class MinStats(Structure):
    _fields_ = [("iteration", c_int32), ("converged", c_int32), ("converged_iteration", c_int32),
                ("convergence_count", c_int32), ("condA", c_int32), ("condB", c_int32),
                ("xB_clamped", c_int32), ("elastic_iterations", c_int32),
                ("mean_h", c_double), ("V0_target", c_double), ("lambda_vol", c_double),
                ("F_surf", c_double), ("F_el", c_double), ("F_chem_excess", c_double),
                ("F_total_excess", c_double), ("F_chem_CNT", c_double), ("F_total_CNT", c_double),
                ("total_interface_sum", c_double), ("total_el_core_sum", c_double),
                ("rms_res", c_double), ("rms_dphi", c_double), ("rms_dY", c_double),
                ("energy_diff_rel", c_double), ("vol_err_rel", c_double),
                ("elastic_relative_residual", c_double)]


class Case(Structure):
    _fields_ = [("params", Params), ("phi", c_void_p), ("xB", c_void_p), ("eta", c_void_p),
                ("phi_out", c_void_p), ("xB_out", c_void_p), ("max_iter", c_int32),
                ("stop_on_convergence", c_int32), ("stats", MinStats), ("status", c_int32), ("pad", c_int32),
                ("seconds", c_double), ("message", ctypes.c_char * 160)]


class Diag(Structure):
    _fields_ = [("vf_precip", c_double), ("mass_xBtot", c_double), ("mean_xB", c_double),
                ("phi_min", c_double), ("phi_max", c_double), ("xB_min", c_double),
                ("xB_max", c_double), ("n_in", c_double), ("n_if", c_double)]


class CkptProvenance(Structure):
    _fields_ = [("zero_mode", ctypes.c_char * 64), ("backend", ctypes.c_char * 64),
                ("composition_mode", ctypes.c_char * 64), ("y_update_mode", ctypes.c_char * 64),
                ("explicit_context", ctypes.c_char * 64), ("reaction_discretization", ctypes.c_char * 64),
                ("elastic_solver_mode", ctypes.c_char * 64), ("initial_state_class", ctypes.c_char * 96),
                ("fixture_manifest_sha256", ctypes.c_char * 96),
                ("profile_library_manifest_sha256", ctypes.c_char * 96),
                ("elastic_solver_fingerprint", ctypes.c_uint64), ("parameter_fingerprint", ctypes.c_uint64)]


class CkptState(Structure):
    _fields_ = [("accepted_step", ctypes.c_uint64), ("nx", c_int32), ("ny", c_int32), ("nz", c_int32),
                ("elastic_present", c_int32), ("dt_code", c_double), ("temperature_K", c_double),
                ("target_mass_code", c_double), ("last_lambda", c_double), ("last_residual_code", c_double),
                ("last_derivative_code", c_double), ("last_iterations", ctypes.c_uint64),
                ("accepted_zero_mode_steps", ctypes.c_uint64), ("elastic_source_field_step", ctypes.c_uint64),
                ("elastic_last_iterations", ctypes.c_uint64), ("elastic_last_relative_residual", c_double),
                ("provenance", CkptProvenance), ("phi", c_void_p), ("Y", c_void_p), ("xB", c_void_p),
                ("dY_dt_prev", c_void_p), ("displacement_k", c_void_p)]


class FnoConfig(Structure):
    _fields_ = [("Nx", c_int32), ("Ny", c_int32), ("Nz", c_int32), ("modes", c_int32), ("layers", c_int32),
                ("pad", c_int32), ("seed", ctypes.c_uint64), ("in_scale", ctypes.c_float * 8),
                ("out_scale", ctypes.c_float * 3), ("pad2", ctypes.c_float)]


class FnoAdam(Structure):
    _fields_ = [("lr", ctypes.c_float), ("beta1", ctypes.c_float), ("beta2", ctypes.c_float),
                ("eps", ctypes.c_float), ("weight_decay", ctypes.c_float), ("clip_norm", ctypes.c_float)]


# (name, restype, argtypes) of every entry point declared in include/pfgb.h
EXPORTS = [
    ("pfgb_params_size", c_size_t, []),
    ("pfgb_params_default", None, [POINTER(Params)]),
    ("pfgb_params_finalize", c_int, [POINTER(Params)]),
    ("pfgb_params_load_file", c_int, [POINTER(Params), c_char_p, c_char_p, c_size_t]),
    ("pfgb_params_set", c_int, [POINTER(Params), c_char_p, c_char_p]),
    ("pfgb_status_string", c_char_p, [c_int]),
    ("pfgb_create", c_int, [POINTER(Params), c_int, POINTER(c_void_p)]),
    ("pfgb_destroy", None, [c_void_p]),
    ("pfgb_last_error", c_char_p, [c_void_p]),
    ("pfgb_set_stream", c_int, [c_void_p, c_void_p]),
    ("pfgb_device_bytes", c_size_t, [c_void_p]),
    ("pfgb_prepare_raw_fields", c_int, [POINTER(Params), c_double, c_void_p, c_void_p, c_void_p,
                                        c_void_p, c_size_t]),
    ("pfgb_load_fields", c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    ("pfgb_load_fields_device", c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    ("pfgb_set_fields", c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    ("pfgb_step", c_int, [c_void_p, c_int, POINTER(StepStats)]),
    ("pfgb_minimize", c_int, [c_void_p, c_int, c_int, POINTER(MinStats)]),
    ("pfgb_batch_minimize", c_int, [POINTER(Case), c_int, c_int, c_int]),
    ("pfgb_init_fields", c_int, [c_void_p]),
    ("pfgb_seed_fields", c_int, [POINTER(Params), c_int, c_void_p, c_void_p]),
    ("pfgb_read_fields", c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    ("pfgb_read_elastic", c_int, [c_void_p, c_void_p, c_void_p]),
    ("pfgb_read_displacement_k", c_int, [c_void_p, c_void_p]),
    ("pfgb_diagnostics", c_int, [c_void_p, POINTER(Diag)]),
    ("pfgb_sync", c_int, [c_void_p]),
    ("pfgb_profile_enable", c_int, [c_void_p, c_int]),
    ("pfgb_profile_launches", ctypes.c_longlong, [c_void_p]),
    ("pfgb_profile_read", c_int, [c_void_p, POINTER(c_char_p), POINTER(c_double), POINTER(c_double),
                                  POINTER(c_int), c_int]),
    ("pfgb_fft3d_r2c", c_int, [c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p]),
    ("pfgb_fft3d_c2r", c_int, [c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p]),
    ("pfgb_fft3d_r2c_noalloc", c_int, [c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p]),
    ("pfgb_fft_y246x6", c_int, [c_int, c_int, c_int, c_int, c_void_p, c_void_p]),
    ("pfgb_tile_report", ctypes.c_size_t, [ctypes.c_char_p, ctypes.c_size_t]),
    ("pfgb_set_tune_copies", None, [c_int]),
    ("pfgb_fnv1a64", ctypes.c_uint64, [c_void_p, c_size_t, ctypes.c_uint64]),
    ("pfgb_parameter_fingerprint", ctypes.c_uint64, [POINTER(Params)]),
    ("pfgb_elastic_solver_fingerprint", ctypes.c_uint64, [POINTER(Params)]),
    ("pfgb_checkpoint_provenance_for", c_int, [POINTER(Params), c_char_p, c_char_p, c_char_p,
                                               POINTER(CkptProvenance)]),
    ("pfgb_checkpoint_write_file", c_int, [c_char_p, POINTER(CkptState)]),
    ("pfgb_checkpoint_peek", c_int, [c_char_p, POINTER(c_int32), POINTER(c_int32), POINTER(c_int32),
                                     POINTER(c_int32), POINTER(c_int32)]),
    ("pfgb_checkpoint_read_file", c_int, [c_char_p, POINTER(CkptProvenance), POINTER(CkptState)]),
    ("pfgb_checkpoint_save", c_int, [c_void_p, c_char_p, c_char_p, c_char_p, c_char_p]),
    ("pfgb_checkpoint_restore", c_int, [c_void_p, c_char_p, c_char_p, c_char_p, c_char_p]),
    ("pfgb_fno_config_default", None, [POINTER(FnoConfig)]),
    ("pfgb_fno_create", c_int, [POINTER(FnoConfig), c_int, POINTER(c_void_p)]),
    ("pfgb_fno_destroy", None, [c_void_p]),
    ("pfgb_fno_set_stream", c_int, [c_void_p, c_void_p]),
    ("pfgb_fno_get_config", c_int, [c_void_p, POINTER(FnoConfig)]),
    ("pfgb_fno_set_scales", c_int, [c_void_p, c_void_p, c_void_p]),
    ("pfgb_fno_num_params", ctypes.c_longlong, [c_void_p]),
    ("pfgb_fno_get_params", c_int, [c_void_p, c_void_p, ctypes.c_longlong]),
    ("pfgb_fno_set_params", c_int, [c_void_p, c_void_p, ctypes.c_longlong]),
    ("pfgb_fno_forward", c_int, [c_void_p, c_void_p, c_void_p]),
    ("pfgb_fno_loss_grad", c_int, [c_void_p, c_void_p, c_void_p, c_int, POINTER(c_double)]),
    ("pfgb_fno_get_grad", c_int, [c_void_p, c_void_p, ctypes.c_longlong]),
    ("pfgb_fno_adam_step", c_int, [c_void_p, POINTER(FnoAdam)]),
    ("pfgb_fno_save", c_int, [c_void_p, c_char_p]),
    ("pfgb_fno_load", c_int, [c_char_p, c_int, c_int, c_int, c_int, POINTER(c_void_p)]),
    ("pfgb_set_warm_start_model", c_int, [c_void_p, c_void_p]),
    ("pfgb_elastic_training_pair", c_int, [c_void_p, c_void_p, c_void_p, POINTER(StepStats)]),
]

_LIB = None


class PfgbError(RuntimeError):
    def __init__(self, status: int, where: str, detail: str = ""):
        self.status = status
        super().__init__(f"{where}: {STATUS.get(status, status)}" + (f" ({detail})" if detail else ""))


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = False) -> ctypes.CDLL:
    """Load libpfgb.so; raises OSError if it is not built (no fallback)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = library_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise OSError(f"pfgb CUDA library not built: {path} (run python -m cuda_sto_pf_gb300.build)")
        _build.build()
    lib = ctypes.CDLL(path)
    for name, res, args in EXPORTS:
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    if lib.pfgb_params_size() != ctypes.sizeof(Params):
        raise OSError(f"pfgb_params size mismatch: C {lib.pfgb_params_size()} vs ctypes {ctypes.sizeof(Params)}")
    _LIB = lib
    return lib


def check(status: int, where: str, ctx=None) -> None:
    if status != 0:
        lib = load()
        detail = lib.pfgb_last_error(ctx).decode(errors="replace") if lib else ""
        raise PfgbError(status, where, detail)


def default_params() -> Params:
    p = Params()
    load().pfgb_params_default(ctypes.byref(p))
    return p


def tile_report() -> str:
    """The generic engine's autotuned tiles in this process (fft_autotune)."""
    L = load()
    n = L.pfgb_tile_report(None, 0)
    buf = ctypes.create_string_buffer(n + 1)
    L.pfgb_tile_report(buf, n + 1)
    return buf.value.decode()


def load_params_file(path: str, p: Params | None = None) -> Params:
    lib = load()
    if p is None:
        p = default_params()
    err = ctypes.create_string_buffer(512)
    st = lib.pfgb_params_load_file(ctypes.byref(p), path.encode(), err, 512)
    if st != 0:
        raise PfgbError(st, "pfgb_params_load_file", err.value.decode(errors="replace"))
    return p


def set_param(p: Params, key: str, value) -> None:
    st = load().pfgb_params_set(ctypes.byref(p), key.encode(), str(value).encode())
    if st != 0:
        raise PfgbError(st, f"pfgb_params_set({key})")


def finalize(p: Params) -> Params:
    check(load().pfgb_params_finalize(ctypes.byref(p)), "pfgb_params_finalize")
    return p
