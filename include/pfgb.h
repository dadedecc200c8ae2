/*
 * pfgb.h — C ABI of the GB300-native phase-field time-stepping library.
 *
 * The library advances the CUDA_STO_PF Ag2Te/PbTe phase-field model
 * (phi Allen-Cahn, eta GP-zone Allen-Cahn, logit-composition Y
 * Cahn-Hilliard, FFT micro-elasticity with heterogeneous stiffness) on one
 * GPU.  Every entry point takes plain pointers and sizes and returns a
 * pfgb_status; nothing calls exit().
 *
 * Which reference interface each entry point replaces (the reference has no
 * library API; its hot path is inline code in main() of main_cuda.cu):
 *   pfgb_params            <- PFParams, pf_params.h:6-702 (hot-path subset)
 *   pfgb_params_default    <- params_default(), main_cuda.cu:15781-16439
 *   pfgb_params_finalize   <- pfparams_refresh_thermo(), main_cuda.cu:15603-15613
 *   pfgb_create            <- device allocation + cuFFT plans + kspace_build_cuda,
 *                             main_cuda.cu:27757-28182, cuda_common.cu:76-109
 *   pfgb_load_fields       <- initial host->device copies, main_cuda.cu:28046-28076
 *                             (fields prepared by load_raw_init_fields,
 *                             main_cuda.cu:2904-2990 -> pfgb_prepare_raw_fields)
 *   pfgb_step              <- one pass of `for (step...)`, main_cuda.cu:28427-31623
 *   pfgb_minimize          <- the same loop with --mode=minimize,
 *                             main_cuda.cu:29264-29750, 32100-32600
 *   pfgb_read_fields       <- device->host copies before VTK/CSV output,
 *                             main_cuda.cu:32760-32820
 *   pfgb_diagnostics       <- gpu_compute_vf_from_h / gpu_reduce_sum_xBtot /
 *                             gpu_reduce_min_max, cuda_kernels.cu:5609-5942
 *   pfgb_fft3d_*           <- cufftExecD2Z/Z2D/R2C/C2R call sites,
 *                             main_cuda.cu:28163-28173 (own kernels, no cuFFT)
 *   pfgb_checkpoint_*      <- pf_zero_mode::write_checkpoint / read_checkpoint
 *                             (pf_zero_mode_checkpoint.h:80-95) and their use
 *                             by main_cuda.cu:27340-28100 (restart) and
 *                             33494-33560 (periodic write); same file format
 *   pfgb_parameter_fingerprint, pfgb_elastic_solver_fingerprint
 *                          <- pf_zero_mode_parameter_fingerprint /
 *                             elastic_solver_parameter_fingerprint,
 *                             main_cuda.cu:4187-4264
 *   pfgb_fno_*, pfgb_set_warm_start_model, pfgb_elastic_training_pair
 *                          <- no counterpart: a learned start for the
 *                             heterogeneous elastic iteration at the
 *                             reference's warm-start point,
 *                             main_cuda.cu:28792-28870
 *
 * Layouts: real fields are C-order [Nx][Ny][Nz] (z fastest, idx=(i*Ny+j)*Nz+k,
 * io_vtk_cuda.h:104-108); spectral fields are the half spectrum
 * [Nx][Ny][Nz/2+1] of interleaved (re,im) pairs, unnormalised forward
 * transform with exp(-i k.x), like cuFFT D2Z/R2C.
 */
#ifndef PFGB_H
#define PFGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PFGB_ABI_VERSION 1

typedef enum pfgb_status {
    PFGB_OK = 0,
    PFGB_ERR_INVALID = 1,        /* bad argument or parameter value        */
    PFGB_ERR_CUDA = 2,           /* a CUDA runtime call failed             */
    PFGB_ERR_NOMEM = 3,          /* device allocation failed               */
    PFGB_ERR_NONCONVERGED = 4,   /* elastic fixed point hit iter_max
                                    (elastic_fail_on_nonconvergence=1)     */
    PFGB_ERR_ZERO_MODE = 5,      /* zero-mode mass solve rejected the step */
    PFGB_ERR_NONFINITE = 6,      /* NaN/Inf residual or field              */
    PFGB_ERR_TIMEOUT = 7,        /* a bounded device wait ran out          */
    PFGB_ERR_UNSUPPORTED = 8,    /* option outside the implemented path    */
    PFGB_ERR_IO = 9              /* a model file could not be read/written */
} pfgb_status;

/* field / transform precision */
enum { PFGB_PREC_FP64 = 0, PFGB_PREC_FP32 = 1 };
/* model_mode (pf_params.h model_mode string) */
enum { PFGB_MODEL_TWO_PHASE = 0, PFGB_MODEL_GP_ZONE = 1 };
/* mode (pf_params.h: 0=dynamics, 1=minimize) */
enum { PFGB_MODE_DYNAMICS = 0, PFGB_MODE_MINIMIZE = 1 };
/* pf_y_update_mode (pf_params.h:345) */
enum { PFGB_Y_LAGGED_RHS = 0, PFGB_Y_STORAGE_EXACT = 1, PFGB_Y_X_TRANSPORT_SPLIT = 2, PFGB_Y_Q_TRANSPORT_SPLIT = 3 };
enum { PFGB_COMPOSITION_LEGACY = 0, PFGB_COMPOSITION_CTOT = 1, PFGB_COMPOSITION_QALPHA = 2 };
enum { PFGB_CONS_FLUX_PAIRWISE_LIMITED = 0, PFGB_CONS_FLUX_BACKWARD_EULER = 1 };
/* gp_y_update_mode (gp_y_update_mode_code, main_cuda.cu:16786-16793) */
enum { PFGB_GP_Y_OLD_RHS = 0, PFGB_GP_Y_PICARD_STORAGE = 1, PFGB_GP_Y_STORAGE_EXACT = 2, PFGB_GP_Y_CONSERVATIVE_RHS = 3 };
enum { PFGB_GP_ETA_LIMITER_OFF = 0, PFGB_GP_ETA_LIMITER_LOCAL_CLIP = 1 };

/*
 * Stiffness tensors are the 21 independent Voigt entries in the reference's
 * argument order 11,12,13,14,15,16,22,23,24,25,26,33,34,35,36,44,45,46,55,56,66
 * (Voigt 4=yz, 5=xz, 6=xy).  Strain 6-vectors are xx,yy,zz,yz,xz,xy.
 */
typedef struct pfgb_params {
    /* grid / time */
    int32_t Nx, Ny, Nz;
    int32_t model_mode;
    int32_t mode;
    int32_t precision;            /* PFGB_PREC_* of phi/eta/Y fields + their FFTs */
    int32_t elastic_precision;    /* PFGB_PREC_* of the elastic solve (ref: FP32) */
    int32_t thermo_convex_extrapolation_enabled;
    double dx, dy, dz, dt;
    /* thermodynamics (dimensionless) */
    double temperature_C;
    double mu_reference_scale;
    double W, kappa_phi, L_phi;
    double D_alpha, D_compound;
    double v_A, v_B;
    double Vm_compound, Vm_alpha_0, dVm_alpha_dxB;
    double Y_clip, xB_eps;
    double elastic_shift_dimless;
    /* elasticity */
    int32_t elastic_enabled;
    int32_t elastic_warm_start_enabled;
    int32_t elastic_residual_control_enabled;
    int32_t elastic_iter_min;
    int32_t elastic_iter_max;
    int32_t elastic_fail_on_nonconvergence;
    /* 1: iterate the increment delta = u - u0 from the warm start u0 (after
       one full evaluation r0 = Phi(u0) - u0, each update is delta <- r0 +
       L delta with only the linear part of the operator); the same iterates
       and residual as the reference's u <- Phi(u) in exact arithmetic, with
       FP32 rounding noise relative to |delta| instead of |u|.  0: the
       reference's form.  No counterpart key in the reference. */
    int32_t elastic_increment_form;
    /* 1: once two earlier steps' solutions exist, start the fixed point from
       the linear extrapolation 2 u^n - u^{n-1} instead of u^n (the
       reference's warm start, main_cuda.cu:28795-28807); it converges to the
       same tolerance from a guess accurate to O(dt^2).  2: once three exist,
       the quadratic 3 u^n - 3 u^{n-1} + u^{n-2}, accurate to O(dt^3); 3:
       once four exist, the cubic 4 u^n - 6 u^{n-1} + 4 u^{n-2} - u^{n-3};
       4: once five exist, the quartic (5, -10, 10, -5, 1); 5: once six
       exist, the quintic (6, -15, 20, -15, 6, -1).  Default 0. */
    int32_t elastic_warm_start_extrapolate;
    /* 1: Chebyshev semi-iteration of the increment fixed point (with
       elastic_increment_form).  The linear part L = -Gamma0 (h dC) is
       self-adjoint in the C0 energy inner product, so its spectrum is real
       and lies in [min(0, -mu_max), max(0, -mu_min)], mu the generalised
       eigenvalues of (dC, C0) (h in [0, 1]).  From those bounds the update
       takes the relaxation 2 / (2 - a - b) and the Chebyshev three-term
       recurrence.  Same fixed point and the same residual test as the
       reference's iteration, in fewer iterations.  No counterpart key in the
       reference; default 0. */
    int32_t elastic_chebyshev;
    /* Bit mask of the elastic-iteration passes whose 246 = 6 x 41
       transforms run their 41-point stage on the tensor cores as a
       split-precision TF32 contraction (three terms, FP32 accumulation;
       tcgen05.mma with the accumulators in tensor memory) instead of direct
       FP32 multiply-adds: 1 the y passes, 2 the x (Green's operator) pass,
       4 the z (h_ij) pass.  A bit applies where that axis is 246 long (x and
       y also with an even Nz/2+1) and the elastic fields are FP32.  No
       counterpart key in the reference (its transforms are cuFFT's);
       default 0. */
    int32_t fft_tensor_cores;
    /* Bits: the generic transform engine (axes other than 246 long) times
       its tile candidates on first use, per kernel, grid shape and device,
       and keeps the fastest for the life of the process: 1 the columns per
       block of the x and y passes (timed as themselves), 2 the rows per
       block of the z passes (timed through a copy op with the same field
       counts); pfgb_tile_report lists them.  0 (default): the fixed rule,
       the largest tile within 112 KiB of shared memory.  No counterpart key
       in the reference. */
    int32_t fft_autotune;
    int32_t pad_fft;
    double elastic_residual_tolerance;
    double elastic_residual_absolute_floor;
    double eps_iso_over_vB;
    double eps00[6];
    double E0[6];
    double S[21];
    double S_p[21];
    /* Y (composition) update options */
    int32_t enable_Y_rhs_previous_time_level;
    int32_t disable_Y_rhs_gamma_term;
    double Y_rhs_term_h_scale;
    /* pf_y_update_mode: PFGB_Y_LAGGED_RHS (the semi-implicit spectral update,
       default) or PFGB_Y_STORAGE_EXACT (two_phase, zero mode off: the
       storage-consistent point update C^{n+1} = C^n + dt div J solved for
       x_alpha, two_phase_storage_exact_Y_update_kernel,
       cuda_kernels.cu:2859-2921); gp_h_alpha_eps is its matrix-storage floor;
       or PFGB_Y_X_TRANSPORT_SPLIT (two_phase, zero mode off: x_alpha advanced
       semi-implicitly with the source div J / (1 - h) where 1 - h is at least
       pf_matrix_storage_floor, stabilised by D_alpha times
       pf_composition_stabilizer_Dalpha_multiplier, main_cuda.cu:30564-30676);
       or PFGB_Y_Q_TRANSPORT_SPLIT (two_phase dynamics, zero mode off: the
       matrix storage q = (1 - h) x_alpha is the conserved coordinate; a local
       phase transfer q -= dh v_B after the phi update (the phi substep is
       rejected where it would leave [0, 1 - h]), explicit transport
       q += dt div J with the matrix-channel mobility (1 - h) M_alpha, a
       sequential local redistribution where transport leaves the bounds, and
       x_alpha = q / (1 - h); main_cuda.cu:27781-27783, 30241-30277,
       30648-30707, 22362-22456, cuda_kernels.cu:2014-2037, 2975-3116) */
    int32_t pf_y_update_mode;
    int32_t pad_y;
    double gp_h_alpha_eps;
    double pf_matrix_storage_floor;
    double pf_composition_stabilizer_Dalpha_multiplier;
    /* GP storage coupling switches (gp_storage_coupling_enabled,
       main_cuda.cu:16767-16772; defaults 1 and 0): gp_zone with
       gp_barrier_only_mode = 0 or enable_legacy_gp_storage_coupling = 1
       conserves xBtot_gp = h_alpha x + h_GP gp_xB_fixed + h_beta; the Y
       update then follows gp_y_update_mode and gp_eta_mass_limiter below. */
    int32_t gp_barrier_only_mode;
    int32_t enable_legacy_gp_storage_coupling;
    /* zero mode (PF_CONSERVED_Y_ZERO_MODE_V1) */
    int32_t zero_mode_enabled;
    int32_t zero_mode_max_iterations;
    double zero_mode_tolerance_relative;
    /* GP zone (model_mode=gp_zone) */
    int32_t gp_elastic_enabled;
    int32_t gp_elastic_active_eta;
    int32_t gp_elastic_active_phi;
    int32_t gp_pad0;
    double gp_xB_fixed, gp_delta_g0;
    double gp_W_eta, gp_kappa_eta, gp_L_eta;
    double gp_M_GP, gp_M_beta;
    double gp_eps_iso, gp_elastic_derivative_scale;
    /* minimize (mode=minimize) */
    int32_t minimize_full_model;
    int32_t minimize_post_projection_iters;
    int32_t minimize_max_iter;
    int32_t minimize_convergence_steps;
    double minimize_dt;
    double minimize_V0;
    double eta_lambda_vol;
    double minimize_xB_max_safe;
    double minimize_rms_dphi_threshold;
    double minimize_rms_dY_threshold;
    double minimize_energy_diff_rel_threshold;
    double minimize_rms_res_threshold;
    double minimize_vol_err_rel_threshold;
    /* provenance keys required in the parameter file (main_cuda.cu:1089-1146),
       used for output naming / physical time, not by the time step */
    int32_t pf_params_schema_version;
    /* zero-mode exact evaluations of an FP32-field run: 0 (default) in
       double-float arithmetic per cell (about 48 bits, FP32 pipe) with FP64
       sums; 1 in FP64 per cell.  FP64-field runs always evaluate in FP64. */
    int32_t zero_mode_fp64_cells;
    double t_real_unit;
    double ic_vf_init_phi, ic_vf_target_phi, ic_phi_iface_w;
    double gamma_Jm2, lambda_sm_m, Vm_alpha_0_phys_m3mol;
    /* initial-condition keys read by minimize: far-field composition
       (ic_23d_xB_out, alias xB_alpha_initial) for the chemical energy
       baseline, and the legacy seed radius / count that set the volume
       target when minimize_V0 <= 0 (compute_effective_vf_target,
       main_cuda.cu:2459-2490) */
    double ic_23d_xB_out;
    double ic_phi_seed_radius;
    double minimize_min_pseudo_time;
    int32_t ic_phi_num_seeds;
    /* starting point of each heterogeneous elastic solve (no counterpart
       key in the reference, which always uses 0):
       0 = the previous step's displacement once one exists (reference);
       1 = the attached model's prediction when no previous solution exists
           (first step, after a load), the previous step's otherwise;
       2 = the model's prediction on every step;
       3 = the homogeneous solution on every step (cold).
       1 and 2 need pfgb_set_warm_start_model. */
    int32_t elastic_warm_start_source;
    /* seeded initial fields (initialize_fields_cuda, main_cuda.cu:15157-15430;
       flags --init-shape, --init-axis-ratio-r*, --init-tilt-*-deg,
       --init-center-shift-*, --init-phi-noise-*, --seed): shape -1 legacy /
       0 sphere / 1 ellipsoid with the axis ratios (normalised to the volume
       of the radius-R sphere); the short axis tilted by (theta, phi) when
       init_use_rotation; every centre shifted; uniform phi noise of
       amplitude init_phi_noise_amp hashed from init_phi_noise_seed (seed
       when 0); seed also places several seeds (srand / rand) */
    int32_t init_shape_mode;
    int32_t init_use_rotation;
    double init_axis_ratio_rx, init_axis_ratio_ry, init_axis_ratio_rz;
    double init_tilt_theta_deg, init_tilt_phi_deg;
    double init_center_shift_x, init_center_shift_y, init_center_shift_z;
    double init_phi_noise_amp;
    uint64_t init_phi_noise_seed;
    uint64_t seed;
    /* PF-only conservative composition modes (pf_composition_mode,
       main_cuda.cu:27784-27792, 28486-28545, 29859-29880, kernels
       cuda_kernels.cu:3117-3288; two_phase dynamics, zero mode off, even
       grid axes): the conserved storage C = q + h v_B (ctot_conservative_split)
       or q = (1 - h) x (qalpha_conservative_local_transaction) is moved by a
       limited pairwise face transfer of the matrix-channel flux on the cell
       grid (six checkerboard sweeps per step, before the elastic solve; the
       backward-Euler damped variant with pf_conservative_flux_strategy =
       PFGB_CONS_FLUX_BACKWARD_EULER), and the phi update is constrained to
       h <= C / v_B; the spectral Y update is not run.  mass_tol and
       max_subcycles are validated as the reference does and not used. */
    int32_t pf_composition_mode;              /* PFGB_COMPOSITION_*        */
    int32_t pf_conservative_flux_strategy;    /* PFGB_CONS_FLUX_*          */
    double pf_conservative_bound_tol;
    double pf_conservative_mass_tol;
    double pf_conservative_beta_support_eps;
    int32_t pf_conservative_max_subcycles;
    /* GP storage coupling (gp_zone dynamics with the coupling on,
       main_cuda.cu:30449-30560, 30587-30628, 30734-30760, 30912-30952):
       gp_y_update_mode PFGB_GP_Y_OLD_RHS (default; the semi-implicit Y update
       with the GP storage source, compute_Y_rhs_gp_kernel,
       cuda_kernels.cu:2361-2430, its h_alpha floored at gp_h_alpha_eps),
       PFGB_GP_Y_CONSERVATIVE_RHS (the same without the floor,
       compute_Y_rhs_gp_conservative_kernel, :2432-2527),
       PFGB_GP_Y_STORAGE_EXACT (the point update of xBtot_gp solved for x,
       gp_storage_exact_Y_update_kernel, :2746-2857) or
       PFGB_GP_Y_PICARD_STORAGE (gp_y_picard_iters fixed-point sweeps of the
       storage update, gp_picard_storage_Y_update_kernel, :3290-3370);
       gp_eta_mass_limiter PFGB_GP_ETA_LIMITER_LOCAL_CLIP caps the GP
       fraction where the recovered matrix composition would leave
       [xB_eps, 1 - xB_eps] (gp_eta_feasibility_and_limiter_kernel,
       :1151-1250), default off. */
    int32_t gp_y_update_mode;
    int32_t gp_eta_mass_limiter;
    int32_t gp_y_picard_iters;
    /* the composition of the mobility in the limiter's second flux: 0
       (default) as the reference computes it, where the buffer of x^n
       (d_xB_prev_r) is the buffer of div J (main_cuda.cu:27858) and so holds
       the first pass's div J by then; 1 = x^n.  No counterpart key in the
       reference. */
    int32_t gp_limiter_flux_from_xn;
    /* y_update_mass_projection_enabled (main_cuda.cu:31085-31140): the
       reference arms its global shift of Y only after a GP-to-beta
       conversion event (main_cuda.cu:30079-30084, not on this path) or in
       the q split, where its target, captured only on such events, stays 0,
       the bracket fails and the shift is 0 (x recomputed from Y, a
       rounding-level change).  So on this path 1 changes nothing beyond
       rounding; it is refused, as in the reference, with the conservative
       composition modes and the zero mode (main_cuda.cu:1719-1727, 24691-24704). */
    int32_t y_update_mass_projection_enabled;
    /* derived by pfgb_params_finalize (pfparams_refresh_thermo) */
    double temperature_K;
    double mu0_compound;
    double xB_eq_matrix;
} pfgb_params;

/* Per-step statistics (elastic_solver_trace.csv / pf_zero_mode_trace.csv). */
typedef struct pfgb_step_stats {
    int32_t step;                     /* steps taken by this context so far   */
    int32_t elastic_iterations;       /* of the last step                     */
    int32_t elastic_converged;
    int32_t elastic_warm_start_used;
    double elastic_relative_residual;
    int32_t elastic_iterations_total; /* summed over the steps of the call    */
    int32_t zero_mode_iterations;
    int32_t zero_mode_newton_steps;
    int32_t zero_mode_bisection_steps;
    double zero_mode_lambda;
    double zero_mode_residual;
    double zero_mode_target_mass;
    double mean_DY;
    /* q_transport_projection_split: the step's phase substep was rejected
       (infeasible local storage transfer, phi kept), and the cells whose
       transport left [0, 1 - h] and went through the local redistribution */
    int32_t q_phase_rejected;
    int32_t q_redistributed_cells;
    /* conservative composition modes: faces whose transfer the storage
       bounds limited, and cells whose phi update the storage constrained */
    int32_t cons_limited_faces;
    int32_t cons_phase_constrained;
    /* GP storage coupling with the local_clip limiter: cells whose eta the
       limiter lowered (both limiter passes of the step) */
    int32_t gp_eta_limited_cells;
    int32_t pad_stats;
} pfgb_step_stats;

/* Minimize iteration statistics (energy_minimize.csv row and the stopping
 * rule, main_cuda.cu:32400-32600).  Energies are the ones evaluated at the
 * start of the last iteration, after its elastic solve, as the reference
 * writes them. */
typedef struct pfgb_min_stats {
    int32_t iteration;            /* minimize iterations taken by the context   */
    int32_t converged;            /* convergence_count reached minimize_convergence_steps */
    int32_t converged_iteration;  /* iteration at which it did (0 if not)       */
    int32_t convergence_count;
    int32_t condA, condB;         /* of the last iteration                      */
    int32_t xB_clamped;           /* the minimize_xB_max_safe clamp fired        */
    int32_t elastic_iterations;   /* of the last iteration                      */
    double mean_h, V0_target, lambda_vol;
    double F_surf, F_el, F_chem_excess, F_total_excess, F_chem_CNT, F_total_CNT;
    double total_interface_sum, total_el_core_sum;
    double rms_res, rms_dphi, rms_dY, energy_diff_rel, vol_err_rel;
    double elastic_relative_residual;
} pfgb_min_stats;

/* One case of a batched minimize sweep (pfgb_batch_minimize). */
typedef struct pfgb_case {
    pfgb_params params;        /* mode = minimize; grids may differ per case   */
    const double *phi, *xB;    /* host raw fields, N = Nx*Ny*Nz float64 each   */
    const double *eta;         /* may be NULL                                  */
    double *phi_out, *xB_out;  /* final fields (host, may be NULL)             */
    int32_t max_iter;          /* minimize iterations (minimize_max_iter if <= 0) */
    int32_t stop_on_convergence;
    pfgb_min_stats stats;      /* out: statistics of the last iteration        */
    int32_t status;            /* out: pfgb_status of the case                 */
    int32_t pad;
    double seconds;            /* out: wall time of the case                   */
    char message[160];         /* out: pfgb_last_error text when status != OK  */
} pfgb_case;

/* Scalar diagnostics of the current state (CSV row, mass ledger). */
typedef struct pfgb_diag {
    double vf_precip;      /* <h(phi)>, gpu_compute_vf_from_h            */
    double mass_xBtot;     /* sum((1-h) xB + h v_B); with the GP storage
                              coupling sum(h_alpha xB + h_GP x_GP + h_beta) */
    double mean_xB;
    double phi_min, phi_max;
    double xB_min, xB_max;
    double n_in;           /* cells with phi > 0.5                       */
    double n_if;           /* interface cells, 0.12 < phi < 0.88
                              (gpu_reduce_sum_N_in_N_if, cuda_kernels.cu:5768) */
} pfgb_diag;

typedef struct pfgb_ctx pfgb_ctx;

/* --- parameters ------------------------------------------------------- */
size_t      pfgb_params_size(void);
void        pfgb_params_default(pfgb_params *p);
/*
 * Apply a `key=value` parameter file (load_pfparams_override_file,
 * main_cuda.cu:22306-22360): '#' comments, unknown keys warned on stderr and
 * ignored, a malformed number is an error, and the required key set
 * (validate_required_pfparams_presence, main_cuda.cu:1089-1146) must be
 * present.  errbuf (may be NULL) receives a one-line reason on failure.
 */
pfgb_status pfgb_params_load_file(pfgb_params *p, const char *path, char *errbuf, size_t errlen);
/* Apply one key (same semantics; returns PFGB_ERR_UNSUPPORTED for an unknown key). */
pfgb_status pfgb_params_set(pfgb_params *p, const char *key, const char *value);
pfgb_status pfgb_params_finalize(pfgb_params *p);
const char *pfgb_status_string(pfgb_status s);

/* --- context ---------------------------------------------------------- */
pfgb_status pfgb_create(const pfgb_params *p, int device, pfgb_ctx **out);
void        pfgb_destroy(pfgb_ctx *ctx);
const char *pfgb_last_error(const pfgb_ctx *ctx);
/* All work of the context is issued on this stream (cudaStream_t, may be 0). */
pfgb_status pfgb_set_stream(pfgb_ctx *ctx, void *cuda_stream);
size_t      pfgb_device_bytes(const pfgb_ctx *ctx);

/*
 * Host-side preparation of raw initial fields, the rules of
 * load_raw_init_fields (main_cuda.cu:2904-2990): phi, eta clamped to [0,1],
 * xB clamped to [xB_eps, 1-xB_eps] and capped at xB_max_safe (NaN = no cap).
 * Returns PFGB_ERR_NONFINITE on NaN/Inf input.  In-place on host buffers.
 */
pfgb_status pfgb_prepare_raw_fields(const pfgb_params *p, double xB_max_safe,
                                    double *phi, double *xB, double *eta,
                                    const double *dYdt_prev, size_t n);

/*
 * Upload the state from HOST buffers (float64, C order, N values each).
 * Y = logit(xB) is formed on the device.  eta and dYdt_prev may be NULL
 * (zero).  Resets the elastic warm state and, when zero mode is on, freezes
 * the target mass sum((1-h) xB + h v_B) (main_cuda.cu:28079-28086).
 */
pfgb_status pfgb_load_fields(pfgb_ctx *ctx, const double *phi, const double *xB,
                             const double *eta, const double *dYdt_prev);
/*
 * Replace the fields from HOST buffers but keep the solver history: the
 * elastic warm state, the zero-mode target mass and the step count (the
 * continuation contract of a checkpoint restart, main_cuda.cu:33494-33560).
 */
pfgb_status pfgb_set_fields(pfgb_ctx *ctx, const double *phi, const double *xB,
                            const double *eta, const double *dYdt_prev);
/* Same as pfgb_load_fields, from DEVICE pointers (float64). */
pfgb_status pfgb_load_fields_device(pfgb_ctx *ctx, const double *d_phi,
                                    const double *d_xB, const double *d_eta,
                                    const double *d_dYdt_prev);

/* Advance nsteps dynamics steps.  stats may be NULL. */
pfgb_status pfgb_step(pfgb_ctx *ctx, int nsteps, pfgb_step_stats *stats);
/* Minimize mode (mode = PFGB_MODE_MINIMIZE, minimize_full_model = 1,
 * two_phase, zero mode off): up to max_iter gradient-flow iterations with
 * the Lagrange volume constraint, post-projection and V0 projection
 * (main_cuda.cu:29264-29750, 32100-32600), stopping early when the
 * reference's convergence rule is met and stop_on_convergence != 0. */
pfgb_status pfgb_minimize(pfgb_ctx *ctx, int max_iter, int stop_on_convergence, pfgb_min_stats *stats);
/* Batched minimize sweep: the reference runs such sweeps (radius, shape and
 * eigenstrain-direction scans) as separate main_cuda jobs.  Here the cases
 * share the device: up to `concurrency` cases run at once, each with its
 * own context and stream, fed from a queue by host threads.  Every case's
 * status lands in cases[i].status; the return value is PFGB_OK when all
 * succeeded, else the first failing status.  No counterpart in the
 * reference's library (it has none); replaces the sweep job scripts. */
pfgb_status pfgb_batch_minimize(pfgb_case *cases, int ncases, int device, int concurrency);

/* Seeded initial fields on the device, as the reference builds them when no
 * raw fields are given (initialize_fields_cuda, main_cuda.cu:15157-15430:
 * init_phi_kernel, apply_phi_noise_kernel, init_xB_Y_from_phi_kernel, the
 * seed placement and the diffuse-interface lever rule for xB outside the
 * seeds), loaded as the context's initial state like pfgb_load_fields
 * (eta zero). */
pfgb_status pfgb_init_fields(pfgb_ctx *ctx);
/* The same fields into HOST buffers (N float64 each), without a context. */
pfgb_status pfgb_seed_fields(const pfgb_params *p, int device, double *phi, double *xB);

/* Read the state back to HOST buffers (float64); any pointer may be NULL. */
pfgb_status pfgb_read_fields(pfgb_ctx *ctx, double *phi, double *xB, double *Y,
                             double *eta, double *dYdt_prev);
/* Stress sigma (6 x N float32, order xx,yy,zz,yz,xz,xy) and total strain. */
pfgb_status pfgb_read_elastic(pfgb_ctx *ctx, float *sigma6, float *strain6);
/* Warm elastic displacement u_k (3 x Nk complex float32 interleaved). */
pfgb_status pfgb_read_displacement_k(pfgb_ctx *ctx, float *u3);

pfgb_status pfgb_diagnostics(pfgb_ctx *ctx, pfgb_diag *d);

/* Synchronise the context's stream. */
pfgb_status pfgb_sync(pfgb_ctx *ctx);

/* --- instrumentation (no reference counterpart; the reference prints
 *     cudaEvent totals only, main_cuda.cu:32634-32660) -------------------- */
/* Enable/disable per-launch CUDA-event timing on the context stream and
 * reset the accumulators and the launch counter. */
pfgb_status pfgb_profile_enable(pfgb_ctx *ctx, int on);
/* Kernel launches issued by the context since the last enable/reset. */
long long   pfgb_profile_launches(const pfgb_ctx *ctx);
/* Per-tag totals: names, milliseconds, algorithmic bytes, launch counts.
 * Returns the number of tags; pass names == NULL to query it. */
int         pfgb_profile_read(pfgb_ctx *ctx, const char **names, double *ms, double *bytes,
                              int *count, int cap);

/* --- standalone 3D transforms on DEVICE buffers (test / tooling) ------ */
/* precision: PFGB_PREC_FP64 (double in, double2 out) or PFGB_PREC_FP32.
 * Unnormalised, same conventions as cuFFT D2Z/Z2D (R2C/C2R).  Both
 * buffers must start on a 16-byte boundary (any cudaMalloc'd pointer
 * does): the line engines copy tiles in 16-byte units.  A misaligned
 * buffer gets PFGB_ERR_INVALID before anything is launched (this also
 * holds for pfgb_fft3d_r2c_noalloc).                                       */
pfgb_status pfgb_fft3d_r2c(int precision, int Nx, int Ny, int Nz,
                           const void *d_in, void *d_out, void *cuda_stream);
pfgb_status pfgb_fft3d_c2r(int precision, int Nx, int Ny, int Nz,
                           const void *d_in, void *d_out, void *cuda_stream);

/* The elastic iteration's y-axis transform of six half spectra, in place,
 * on the 246 = 6 x 41 engine (test / tooling; no reference counterpart,
 * its transforms are cuFFT's): d_spec6 holds six arrays of Nx x 246 x NzC
 * interleaved complex float one after another (NzC even, 16-byte aligned),
 * dir -1 forward (exp(-i k.x)), +1 inverse, unnormalised.  tensor_cores != 0
 * runs the 41-point stage on the tensor cores (split-precision TF32), as
 * fft_tensor_cores bit 1 does in the solver. */
pfgb_status pfgb_fft_y246x6(int tensor_cores, int dir, int Nx, int NzC, void *d_spec6, void *cuda_stream);

/* The tiles the autotuner (fft_autotune) has chosen in this process, one
 * line each: the pass, the axis length and grid extents, the chosen tile
 * and its time, and the fixed rule's tile and time.  Writes at most len
 * bytes (NUL-terminated) and returns the length of the full report. */
size_t pfgb_tile_report(char *buf, size_t len);
/* How many copies of a tile candidate the autotuner times at once, each on
 * its own stream and arrays (1 to 16; default 1): the number of cases that
 * will share the device, so that tiles are chosen for throughput under that
 * sharing.  pfgb_batch_minimize sets it to its concurrency while it tunes. */
void pfgb_set_tune_copies(int copies);

/* --- allocation-free forward transform -------------------------------- */
/* No counterpart in the reference (its transforms go through cuFFT plans
 * that own their work areas).  Same result as pfgb_fft3d_r2c, but the call
 * allocates no device memory and never synchronises: the per-axis twiddle
 * tables are written into a fixed static device array of
 * PFGB_NOALLOC_SCRATCH_BYTES, one table per axis, each rounded up to 256
 * bytes: sizeof(complex) * (Nx + Ny + Nz) plus padding, i.e. 16 bytes per
 * point of Nx+Ny+Nz in FP64 and 8 in FP32.  Larger requests (for example
 * FP64 with Nx+Ny+Nz above 2048) return PFGB_ERR_INVALID with a message in
 * pfgb_last_error(NULL); nothing is launched then.
 *
 * For callers that cannot allocate on the device: a process whose HBM is
 * already reserved by its own pool allocator, or a stream pipeline that
 * must not stall, since cudaMalloc/cudaFree can synchronise the device.
 *
 * Nothing in the scratch array has to start at zero: each call rewrites the
 * tables it uses, on cuda_stream, before the transform reads them.  The
 * first call on a device (the current device of the calling thread) looks
 * up the array's address on that device and may load the module; make
 * that first call before any stream capture.  All calls on one device share
 * the one array, so calls that overlap in time (other streams, other host
 * threads) race on it: order them on one stream or synchronise between
 * them. */
#define PFGB_NOALLOC_SCRATCH_BYTES 32768
pfgb_status pfgb_fft3d_r2c_noalloc(int precision, int Nx, int Ny, int Nz,
                                   const void *d_in, void *d_out, void *cuda_stream);

/* --- zero-mode checkpoints in the reference's file format ----------------
 * V3 (no elastic state) and V4 (with the elastic warm state u_k) are
 * written; V2, V3 and V4 are read.  The provenance is a restart identity:
 * a file whose selectors, identities or fingerprints differ from the
 * expected ones is rejected before any field is returned, and so is a file
 * whose payload checksum (FNV-1a 64) does not match.  Text fields are
 * NUL-terminated; selectors hold at most 63 characters, identities 95. */
typedef struct pfgb_checkpoint_provenance {
    char zero_mode[64];                 /* PF_CONSERVED_Y_ZERO_MODE_V1           */
    char backend[64];                   /* HOST_NEWTON_BISECTION_V1              */
    char composition_mode[64];          /* legacy                                */
    char y_update_mode[64];             /* lagged_rhs                            */
    char explicit_context[64];          /* SM_EXPLICIT_CONTEXT_N_V1              */
    char reaction_discretization[64];   /* SM_TANGENT_N_V1                       */
    char elastic_solver_mode[64];       /* ELASTIC_WARM_START_RESIDUAL_V1 or
                                           ELASTIC_RUNTIME_STATE_NOT_REQUIRED    */
    char initial_state_class[96];       /* --pf-initial-state-class (default
                                           LEGACY_UNSPECIFIED), and the two
                                           manifest hashes likewise              */
    char fixture_manifest_sha256[96];
    char profile_library_manifest_sha256[96];
    uint64_t elastic_solver_fingerprint;   /* 0 without the accelerated solver */
    uint64_t parameter_fingerprint;
} pfgb_checkpoint_provenance;

typedef struct pfgb_checkpoint_state {
    uint64_t accepted_step;
    int32_t nx, ny, nz;
    int32_t elastic_present;            /* 1: V4 with the warm state            */
    double dt_code, temperature_K;
    /* zero-mode runtime state */
    double target_mass_code, last_lambda, last_residual_code, last_derivative_code;
    uint64_t last_iterations, accepted_zero_mode_steps;
    /* elastic warm state: the converged u_k used at the start of step
       accepted_step, i.e. of the fields after step accepted_step - 1 */
    uint64_t elastic_source_field_step, elastic_last_iterations;
    double elastic_last_relative_residual;
    pfgb_checkpoint_provenance provenance;
    /* caller-owned host buffers: N = nx*ny*nz float64 each, and
       6 * nx*ny*(nz/2+1) floats (ux_k | uy_k | uz_k, interleaved re/im) */
    double *phi, *Y, *xB, *dY_dt_prev;
    float *displacement_k;
} pfgb_checkpoint_state;

uint64_t pfgb_fnv1a64(const void *data, size_t size, uint64_t seed);
uint64_t pfgb_parameter_fingerprint(const pfgb_params *p);
uint64_t pfgb_elastic_solver_fingerprint(const pfgb_params *p);
/* The provenance the reference builds for these parameters
 * (main_cuda.cu:24721-24743); NULL identities mean LEGACY_UNSPECIFIED. */
pfgb_status pfgb_checkpoint_provenance_for(const pfgb_params *p, const char *initial_state_class,
                                           const char *fixture_manifest_sha256,
                                           const char *profile_library_manifest_sha256,
                                           pfgb_checkpoint_provenance *out);
/* Host-buffer level: validate and write atomically (<path>.tmp, rename). */
pfgb_status pfgb_checkpoint_write_file(const char *path, const pfgb_checkpoint_state *state);
/* Header only: version (2, 3, 4), grid and whether the elastic state is present. */
pfgb_status pfgb_checkpoint_peek(const char *path, int32_t *version, int32_t *nx, int32_t *ny, int32_t *nz,
                                 int32_t *elastic_present);
/* Read into the caller's buffers; state->nx/ny/nz must give the file's grid. */
pfgb_status pfgb_checkpoint_read_file(const char *path, const pfgb_checkpoint_provenance *expected,
                                      pfgb_checkpoint_state *state);
/* Context level (zero mode on, two_phase): write the state after the last
 * step (V4 when the accelerated elastic solver runs), or restore one --
 * fields, zero-mode target and runtime, the elastic warm state and the step
 * count -- after checking grid, dt and temperature and that the restored
 * field's mass ledger matches the frozen target to 1e-12 relative
 * (main_cuda.cu:27342-27365, 28069-28100). */
pfgb_status pfgb_checkpoint_save(pfgb_ctx *ctx, const char *path, const char *initial_state_class,
                                 const char *fixture_manifest_sha256,
                                 const char *profile_library_manifest_sha256);
pfgb_status pfgb_checkpoint_restore(pfgb_ctx *ctx, const char *path, const char *initial_state_class,
                                    const char *fixture_manifest_sha256,
                                    const char *profile_library_manifest_sha256);

/* --- learned start of the heterogeneous elastic iteration ------------- */
/* No counterpart in the reference, which starts each solve from the
 * previous step's displacement (main_cuda.cu:28792-28870).  A Fourier
 * neural operator (FNO-3d, Li et al. 2021: lift 8 -> 32, `layers` spectral
 * layers of width 32 keeping `modes` modes per axis, GELU, projection
 * 32 -> 64 -> 3) maps the 8 input channels
 *     phi, eta, eps0_xx, eps0_yy, eps0_zz, eps0_yz, eps0_xz, eps0_xy
 * (the eigenstrain field the elastic solve sees) to the heterogeneous
 * displacement correction u - u_hom (3 channels, the real-space
 * displacement in grid units of the solver's u).  The solver adds the
 * prediction to the homogeneous solution and then runs the plain fixed
 * point to its residual tolerance: the model moves the starting point
 * only.  Weights are bfloat16 (float32 master copy for training),
 * arithmetic float32.  All tensors are DEVICE float32, channel-major
 * [C][Nx][Ny][Nz]. */
#define PFGB_FNO_WIDTH 32
#define PFGB_FNO_HIDDEN 64
#define PFGB_FNO_IN 8
#define PFGB_FNO_OUT 3
typedef struct pfgb_fno pfgb_fno;
typedef struct pfgb_fno_config {
    int32_t Nx, Ny, Nz;
    int32_t modes;            /* retained modes per axis; 2*modes <= Nx, Ny, Nz */
    int32_t layers;           /* spectral layers                              */
    int32_t pad;
    uint64_t seed;            /* initial weights                              */
    float in_scale[PFGB_FNO_IN];    /* inputs are multiplied by these first  */
    float out_scale[PFGB_FNO_OUT];  /* outputs are multiplied by these last  */
    float pad2;
} pfgb_fno_config;
typedef struct pfgb_fno_adam {
    float lr, beta1, beta2, eps;
    float weight_decay;       /* decoupled (AdamW)                            */
    float clip_norm;          /* global gradient-norm clip; 0 = off           */
} pfgb_fno_adam;

/* Defaults: 128^3, 12 modes, 4 layers, unit scales. */
void pfgb_fno_config_default(pfgb_fno_config *cfg);
pfgb_status pfgb_fno_create(const pfgb_fno_config *cfg, int device, pfgb_fno **out);
void pfgb_fno_destroy(pfgb_fno *fno);
pfgb_status pfgb_fno_set_stream(pfgb_fno *fno, void *cuda_stream);
pfgb_status pfgb_fno_get_config(const pfgb_fno *fno, pfgb_fno_config *cfg);
pfgb_status pfgb_fno_set_scales(pfgb_fno *fno, const float *in_scale, const float *out_scale);
/* Flat float32 parameter vector, in order: P[32][8] p[32], per layer
 * W[32][32] b[32] R[32 in][32 out][4 modes^3][re,im], then Q1[64][32]
 * q1[64] Q2[3][64] q2[3].  Mode index = (jx*2m + jy)*m + kz with jx, jy
 * in [0, 2m) (j < m: wavenumber j, else N - 2m + j) and kz in [0, m). */
long long pfgb_fno_num_params(const pfgb_fno *fno);
pfgb_status pfgb_fno_get_params(pfgb_fno *fno, float *host, long long n);
pfgb_status pfgb_fno_set_params(pfgb_fno *fno, const float *host, long long n);
/* d_in [8][N] -> d_out [3][N] on the model's stream. */
pfgb_status pfgb_fno_forward(pfgb_fno *fno, const float *d_in, float *d_out);
/* Forward and backward of the loss sum (y - t)^2 / sum t^2; the gradient
 * goes to the model's gradient buffer (added to it when accumulate != 0).
 * loss may be NULL (no synchronisation then). */
pfgb_status pfgb_fno_loss_grad(pfgb_fno *fno, const float *d_in, const float *d_target,
                               int accumulate, double *loss);
pfgb_status pfgb_fno_get_grad(pfgb_fno *fno, float *host, long long n);
pfgb_status pfgb_fno_adam_step(pfgb_fno *fno, const pfgb_fno_adam *opt);
/* Model file: header, scales and the float32 parameter vector.  load may
 * place the model on another grid (Nx, Ny, Nz > 0) with the same weights. */
pfgb_status pfgb_fno_save(pfgb_fno *fno, const char *path);
pfgb_status pfgb_fno_load(const char *path, int Nx, int Ny, int Nz, int device, pfgb_fno **out);

/* Attach (or with NULL detach) the model used by elastic_warm_start_source
 * 1 and 2.  The model must be on the context's grid and device; it stays
 * owned by the caller and must outlive its use by the context. */
pfgb_status pfgb_set_warm_start_model(pfgb_ctx *ctx, pfgb_fno *fno);
/* Training pair from the context's current fields: one cold heterogeneous
 * elastic solve to the residual tolerance, then d_in8 [8][N] = the model
 * inputs and d_target3 [3][N] = u - u_hom in real space (DEVICE float32).
 * The fields are not advanced; the solution becomes the context's warm
 * state, as after a step.  stats (may be NULL) gets the iteration count. */
pfgb_status pfgb_elastic_training_pair(pfgb_ctx *ctx, float *d_in8, float *d_target3,
                                       pfgb_step_stats *stats);

#ifdef __cplusplus
}
#endif
#endif /* PFGB_H */
