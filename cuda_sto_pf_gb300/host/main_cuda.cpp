// main_cuda — command-line driver of the pfgb library with the reference
// main_cuda's invocation, parameter file and output layout for the dynamics
// path (main_cuda.cu main(), :22500-34800).  Host C++ over the C ABI only.
//
//   main_cuda Nx Ny Nz dt nsteps out_every csv_out_every elastic(0/1) \
//       --pf-param-file <path> --init-mode raw_fields --init-phi-raw <f> \
//       --init-xB-raw <f> [--init-eta-raw <f>] [--init-dY-dt-prev-raw <f>] \
//       [--init-meta <json>] [--pf-zero-mode PF_CONSERVED_Y_ZERO_MODE_V1] ...
//
// Outputs (CUDA_STO_RESULTS_ROOT, default Results/):
//   <chel|ch>_T%.0f_cuda_NxxNyxNz_dt%.3g_steps%d_xB%.3f/pf_input.params
//   .../<case tag>/pf_input.params, vf_precip_vs_time_<tag>.csv,
//   phi|xB|xBtot|eta VTK (init, every out_every steps, final),
//   elastic_solver_trace.csv, pf_zero_mode_trace.csv,
//   performance_summary.json, summary.txt
// Exit status: 0 success, 2 invalid input or solver failure, 1 CUDA error.
#include <sys/stat.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <string>
#include <thread>
#include <vector>

#include "pfgb.h"

namespace {

// field output: ASCII VTK (the reference's format and the default), legacy
// binary VTK (big-endian float64, the same point order), or raw float64 in
// the C order [Nx][Ny][Nz] that --init-*-raw reads
enum class OutFmt { VtkAscii, VtkBinary, Raw };
OutFmt g_out_fmt = OutFmt::VtkAscii;

struct Cli {
    int pos_Nx = -1, pos_Ny = -1, pos_Nz = -1, nsteps = 100, out_every = 100, csv_out_every = 10;
    int pos_elastic = -1;
    double pos_dt = NAN;
    std::string mode = "dynamics";
    std::string param_file, init_mode, init_phi, init_xB, init_eta, init_dYdt, init_meta, case_tag;
    int elastic = -1;
    double temperature_C = NAN;
    std::string zero_mode;
    double zm_tol = NAN;
    int zm_maxit = -1;
    bool prev_level = false, no_gamma = false;
    double h_scale = NAN;
    int precision = PFGB_PREC_FP64;
    int device = 0;
    std::string warm_model;   // learned start of the elastic iteration (no reference counterpart)
    int warm_source = -1;
    // zero-mode checkpoints (main_cuda.cu:22715-22760)
    // seeded initialisation flags, applied as parameter keys (main_cuda.cu:23915-23972)
    std::vector<std::pair<std::string, std::string>> param_sets;
    bool tilt_given = false;
    double radius_nm = NAN;
    int ckpt_every = 0;
    std::string ckpt_path, restart_from;
    std::string isc = "LEGACY_UNSPECIFIED", fsha = "LEGACY_UNSPECIFIED", psha = "LEGACY_UNSPECIFIED";
    // minimize
    bool min_full = false;
    int min_max_iter = -1, min_conv_steps = -1, min_post_iters = -1;
    double min_dt = NAN, V0 = NAN, eta_lambda = NAN, thr_dphi = NAN, thr_dY = NAN, thr_res = NAN, thr_vol = NAN,
           thr_E = NAN, min_pt = NAN, xB_max_safe = NAN, radius = NAN;
    // continuation from ASCII VTK (--mode=minimize-continue, --continue-phi-vtk,
    // main_cuda.cu:22752-22770, 23770-23780)
    bool cont = false;
    std::string cont_phi, cont_xB;
};

void usage() {
    printf("Usage (positional, legacy):\n"
           "  ./main_cuda Nx Ny Nz dt nsteps out_every csv_out_every elastic_enabled(0/1)\n"
           "    dt is a fallback only: the parameter file's dt wins.\n"
           "\nFlags:\n"
           "  --mode=dynamics|dynamics-continue|minimize|minimize-continue\n"
           "  --continue-phi-vtk <path>       continuation: load phi from ASCII VTK\n"
           "  --continue-xB-vtk <path>        continuation: optional xB ASCII VTK (else rebuilt from phi)\n"
           "  --minimize-full-model           minimize with chemistry + diffusion + volume constraint\n"
           "  --minimize-max-iter <n>  --minimize-dt <dt>  --V0 <v>  --eta-lambda-vol <v>\n"
           "  --minimize-rms-dphi-threshold <v>  --minimize-rms-dY-threshold <v>\n"
           "  --minimize-rms-res-threshold <v>   --minimize-vol-err-rel-threshold <v>\n"
           "  --minimize-energy-diff-rel-threshold <v>  --minimize-convergence-steps <n>\n"
           "  --minimize-post-projection-iters <n>  --minimize-min-pseudo-time <t>\n"
           "  --minimize-xB-max-safe <v>  --radius <r>  (seed radius: V0 target when V0 <= 0)\n"
           "  --pf-param-file <path>          required: complete physical PF inputs (key=value)\n"
           "  --elastic 0|1                   override elastic\n"
           "  --temperature-C <val>\n"
           "  --init-mode raw_fields          initialize from raw phi/xB[/eta][/dY_dt_prev] fields\n"
           "                                  (without it: seeded fields, --radius / --radius-phys-nm,\n"
           "                                  --init-shape sphere|ellipsoid, --init-axis-ratio-r{x,y,z},\n"
           "                                  --init-tilt-{theta,phi}-deg, --init-center-shift-{x,y,z},\n"
           "                                  --init-phi-noise-amp/-seed, --seed, --ic-23d-xB-out)\n"
           "  --init-phi-raw <path>           float64, C order, idx=i*(Ny*Nz)+j*Nz+k\n"
           "  --init-xB-raw <path>\n"
           "  --init-eta-raw <path>           optional (default zero)\n"
           "  --init-dY-dt-prev-raw <path>    optional (default zero history)\n"
           "  --init-meta <path>              init_meta.json (xB_max_safe, grid)\n"
           "  --init-case-tag <tag>           case subdirectory name (default raw_fields_relax)\n"
           "  --pf-zero-mode OFF|PF_CONSERVED_Y_ZERO_MODE_V1\n"
           "  --pf-zero-mode-tol-rel <value>  default 1e-12\n"
           "  --pf-zero-mode-max-iter <n>     default 24\n"
           "  --enable-Y-rhs-previous-time-level\n"
           "  --disable-Y-rhs-gamma-term\n"
           "  --Y-rhs-term-h-scale <s>\n"
           "  --precision fp64|fp32           field precision (default fp64, as the reference)\n"
           "  --device <n>                    CUDA device ordinal\n"
           "  --pf-checkpoint-every <n>       zero-mode checkpoint every n steps and at the end\n"
           "  --pf-checkpoint-path <f>        checkpoint file (V4 with the elastic warm state, else V3)\n"
           "  --pf-restart-from <f>           continue from a zero-mode checkpoint\n"
           "  --pf-initial-state-class <s>  --pf-fixture-manifest-sha256 <s>\n"
           "  --pf-profile-library-manifest-sha256 <s>   restart identity (default LEGACY_UNSPECIFIED)\n"
           "  --output-format vtk|vtk-binary|raw  field files: ASCII VTK (default), legacy binary VTK\n"
           "                                  (big-endian float64) or raw float64 C-order (*.raw)\n"
           "  --elastic-warm-start-model <f>  model file (pfgb_fno_save) for the elastic start\n"
           "  --elastic-warm-start-source <n> 0 previous step (default), 1 model at cold starts,\n"
           "                                  2 model every step, 3 cold every step\n");
}

// "--name value" or "--name=value"; advances i past a separate value
const char *flag_value(int argc, char **argv, int *i, const char *name) {
    const size_t n = strlen(name);
    const char *a = argv[*i];
    if (strncmp(a, name, n) != 0) return nullptr;
    if (a[n] == '=') return a + n + 1;
    if (a[n] != '\0') return nullptr;
    if (*i + 1 >= argc) {
        fprintf(stderr, "[fatal] %s needs a value\n", name);
        exit(2);
    }
    return argv[++*i];
}

bool to_double(const char *s, double *v) {
    char *e = nullptr;
    *v = strtod(s, &e);
    return e != s && *e == '\0' && std::isfinite(*v);
}
bool to_int(const char *s, int *v) {
    char *e = nullptr;
    long x = strtol(s, &e, 10);
    if (e == s || *e != '\0') return false;
    *v = (int)x;
    return true;
}
[[noreturn]] void bad(const char *flag, const char *val) {
    fprintf(stderr, "[fatal] invalid value for %s: %s\n", flag, val);
    exit(2);
}

Cli parse(int argc, char **argv) {
    Cli c;
    // positional arguments sit at fixed places (main_cuda.cu:22527-22534)
    auto posi = [&](int k, int *dst) {
        if (argc > k && argv[k][0] != '-') *dst = atoi(argv[k]);
    };
    posi(1, &c.pos_Nx); posi(2, &c.pos_Ny); posi(3, &c.pos_Nz);
    if (argc > 4 && argv[4][0] != '-') c.pos_dt = atof(argv[4]);
    posi(5, &c.nsteps); posi(6, &c.out_every); posi(7, &c.csv_out_every); posi(8, &c.pos_elastic);
    for (int i = 1; i < argc; ++i) {
        const char *a = argv[i];
        if (a[0] != '-') continue;
        const char *v;
        if (!strcmp(a, "--help") || !strcmp(a, "-h")) { usage(); exit(0); }
        else if (!strncmp(a, "--mode=", 7)) c.mode = a + 7;
        else if ((v = flag_value(argc, argv, &i, "--mode"))) c.mode = v;
        else if ((v = flag_value(argc, argv, &i, "--continue-phi-vtk"))) { c.cont_phi = v; c.cont = true; }
        else if ((v = flag_value(argc, argv, &i, "--continue-xB-vtk"))) c.cont_xB = v;
        else if ((v = flag_value(argc, argv, &i, "--pf-param-file"))) c.param_file = v;
        else if ((v = flag_value(argc, argv, &i, "--elastic"))) { if (!to_int(v, &c.elastic)) bad(a, v); }
        else if ((v = flag_value(argc, argv, &i, "--temperature-C"))) { if (!to_double(v, &c.temperature_C)) bad(a, v); }
        else if ((v = flag_value(argc, argv, &i, "--init-mode"))) c.init_mode = v;
        else if ((v = flag_value(argc, argv, &i, "--init-phi-raw"))) c.init_phi = v;
        else if ((v = flag_value(argc, argv, &i, "--init-xB-raw"))) c.init_xB = v;
        else if ((v = flag_value(argc, argv, &i, "--init-eta-raw"))) c.init_eta = v;
        else if ((v = flag_value(argc, argv, &i, "--init-dY-dt-prev-raw"))) c.init_dYdt = v;
        else if ((v = flag_value(argc, argv, &i, "--init-meta"))) c.init_meta = v;
        else if ((v = flag_value(argc, argv, &i, "--init-case-tag"))) c.case_tag = v;
        else if ((v = flag_value(argc, argv, &i, "--pf-zero-mode-tol-rel"))) { if (!to_double(v, &c.zm_tol)) bad(a, v); }
        else if ((v = flag_value(argc, argv, &i, "--pf-zero-mode-max-iter"))) { if (!to_int(v, &c.zm_maxit)) bad(a, v); }
        else if ((v = flag_value(argc, argv, &i, "--pf-zero-mode"))) c.zero_mode = v;
        else if (!strcmp(a, "--enable-Y-rhs-previous-time-level")) c.prev_level = true;
        else if (!strcmp(a, "--disable-Y-rhs-gamma-term")) c.no_gamma = true;
        else if ((v = flag_value(argc, argv, &i, "--Y-rhs-term-h-scale"))) { if (!to_double(v, &c.h_scale)) bad(a, v); }
        else if ((v = flag_value(argc, argv, &i, "--precision"))) {
            if (!strcmp(v, "fp64")) c.precision = PFGB_PREC_FP64;
            else if (!strcmp(v, "fp32")) c.precision = PFGB_PREC_FP32;
            else bad(a, v);
        }
        else if ((v = flag_value(argc, argv, &i, "--device"))) { if (!to_int(v, &c.device)) bad(a, v); }
        else if ((v = flag_value(argc, argv, &i, "--pf-checkpoint-every")) ||
                 (v = flag_value(argc, argv, &i, "--pf_checkpoint_every"))) { if (!to_int(v, &c.ckpt_every)) bad(a, v); }
        else if ((v = flag_value(argc, argv, &i, "--pf-checkpoint-path")) ||
                 (v = flag_value(argc, argv, &i, "--pf_checkpoint_path"))) c.ckpt_path = v;
        else if ((v = flag_value(argc, argv, &i, "--pf-restart-from")) ||
                 (v = flag_value(argc, argv, &i, "--pf_restart_from"))) c.restart_from = v;
        else if ((v = flag_value(argc, argv, &i, "--pf-initial-state-class")) ||
                 (v = flag_value(argc, argv, &i, "--pf_initial_state_class"))) c.isc = v;
        else if ((v = flag_value(argc, argv, &i, "--pf-fixture-manifest-sha256")) ||
                 (v = flag_value(argc, argv, &i, "--pf_fixture_manifest_sha256"))) c.fsha = v;
        else if ((v = flag_value(argc, argv, &i, "--pf-profile-library-manifest-sha256")) ||
                 (v = flag_value(argc, argv, &i, "--pf_profile_library_manifest_sha256"))) c.psha = v;
        else if ((v = flag_value(argc, argv, &i, "--output-format"))) {
            if (!strcmp(v, "vtk")) g_out_fmt = OutFmt::VtkAscii;
            else if (!strcmp(v, "vtk-binary")) g_out_fmt = OutFmt::VtkBinary;
            else if (!strcmp(v, "raw")) g_out_fmt = OutFmt::Raw;
            else bad(a, v);
        }
        else if ((v = flag_value(argc, argv, &i, "--elastic-warm-start-model"))) c.warm_model = v;
        else if ((v = flag_value(argc, argv, &i, "--elastic-warm-start-source"))) {
            if (!to_int(v, &c.warm_source) || c.warm_source < 0 || c.warm_source > 3) bad(a, v);
        }
        else if (!strcmp(a, "--minimize-full-model")) c.min_full = true;
        else if ((v = flag_value(argc, argv, &i, "--minimize-max-iter"))) { if (!to_int(v, &c.min_max_iter)) bad(a, v); }
        else if ((v = flag_value(argc, argv, &i, "--minimize-dt"))) { if (!to_double(v, &c.min_dt)) bad(a, v); }
        else if ((v = flag_value(argc, argv, &i, "--V0"))) { if (!to_double(v, &c.V0)) bad(a, v); }
        else if ((v = flag_value(argc, argv, &i, "--eta-lambda-vol"))) { if (!to_double(v, &c.eta_lambda)) bad(a, v); }
        else if ((v = flag_value(argc, argv, &i, "--minimize-rms-dphi-threshold"))) { if (!to_double(v, &c.thr_dphi)) bad(a, v); }
        else if ((v = flag_value(argc, argv, &i, "--minimize-rms-dY-threshold")) ||
                 (v = flag_value(argc, argv, &i, "--minimize-rms-dy-threshold"))) { if (!to_double(v, &c.thr_dY)) bad(a, v); }
        else if ((v = flag_value(argc, argv, &i, "--minimize-rms-res-threshold"))) { if (!to_double(v, &c.thr_res)) bad(a, v); }
        else if ((v = flag_value(argc, argv, &i, "--minimize-vol-err-rel-threshold"))) { if (!to_double(v, &c.thr_vol)) bad(a, v); }
        else if ((v = flag_value(argc, argv, &i, "--minimize-energy-diff-rel-threshold"))) { if (!to_double(v, &c.thr_E)) bad(a, v); }
        else if ((v = flag_value(argc, argv, &i, "--minimize-convergence-steps"))) { if (!to_int(v, &c.min_conv_steps)) bad(a, v); }
        else if ((v = flag_value(argc, argv, &i, "--minimize-post-projection-iters"))) { if (!to_int(v, &c.min_post_iters) || c.min_post_iters < 0) bad(a, v); }
        else if ((v = flag_value(argc, argv, &i, "--minimize-min-pseudo-time"))) { if (!to_double(v, &c.min_pt)) bad(a, v); }
        else if ((v = flag_value(argc, argv, &i, "--minimize-xB-max-safe"))) { if (!to_double(v, &c.xB_max_safe)) bad(a, v); }
        else if ((v = flag_value(argc, argv, &i, "--radius"))) { if (!to_double(v, &c.radius) || c.radius < 0) bad(a, v); }
        else if ((v = flag_value(argc, argv, &i, "--radius-phys-nm"))) { if (!to_double(v, &c.radius_nm) || c.radius_nm < 0) bad(a, v); }
        else if ((v = flag_value(argc, argv, &i, "--pf_y_update_mode")) ||
                 (v = flag_value(argc, argv, &i, "--pf-y-update-mode")))   // main_cuda.cu:23410-23414
            c.param_sets.push_back({"pf_y_update_mode", v});
        else if ((v = flag_value(argc, argv, &i, "--pf_composition_mode")) ||
                 (v = flag_value(argc, argv, &i, "--pf-composition-mode")))   // main_cuda.cu:23415-23419
            c.param_sets.push_back({"pf_composition_mode", v});
        else if ((v = flag_value(argc, argv, &i, "--gp-y-update-mode")) ||
                 (v = flag_value(argc, argv, &i, "--gp_y_update_mode")))   // main_cuda.cu:24156-24166
            c.param_sets.push_back({"gp_y_update_mode", v});
        else if ((v = flag_value(argc, argv, &i, "--y-update-mass-projection-enabled")))   // main_cuda.cu:24218-24221
            c.param_sets.push_back({"y_update_mass_projection_enabled", v});
        else if ((v = flag_value(argc, argv, &i, "--gp-barrier-only-mode")))   // main_cuda.cu:24293-24296
            c.param_sets.push_back({"gp_barrier_only_mode", v});
        else if ((v = flag_value(argc, argv, &i, "--enable-legacy-gp-storage-coupling")))   // :24297-24300
            c.param_sets.push_back({"enable_legacy_gp_storage_coupling", v});
        else if ((v = flag_value(argc, argv, &i, "--pf_conservative_flux_strategy")) ||
                 (v = flag_value(argc, argv, &i, "--pf-conservative-flux-strategy")))   // main_cuda.cu:23420-23425
            c.param_sets.push_back({"pf_conservative_flux_strategy", v});
        else if ((v = flag_value(argc, argv, &i, "--init-shape"))) {
            if (!strcmp(v, "sphere")) c.param_sets.push_back({"init_shape_mode", "0"});
            else if (!strcmp(v, "ellipsoid")) c.param_sets.push_back({"init_shape_mode", "1"});
            else bad(a, v);
        }
        else if (!strncmp(a, "--init-axis-ratio-r", 19) || !strncmp(a, "--init-center-shift-", 20) ||
                 !strncmp(a, "--init-tilt-", 12) || !strncmp(a, "--init-phi-noise-", 17) ||
                 !strcmp(a, "--seed") || !strncmp(a, "--seed=", 7) || !strncmp(a, "--ic-23d-xB-out", 15)) {
            // --init-axis-ratio-rx -> init_axis_ratio_rx, --ic-23d-xB-out -> ic_23d_xB_out, ...
            std::string flag = a;
            const size_t eq = flag.find('=');
            if (eq != std::string::npos) flag = flag.substr(0, eq);
            v = flag_value(argc, argv, &i, flag.c_str());
            std::string key = flag.substr(2);
            for (char &ch : key) if (ch == '-') ch = '_';
            c.param_sets.push_back({key, v ? v : ""});
            if (!strncmp(key.c_str(), "init_tilt_", 10)) c.tilt_given = true;
        }
        else fprintf(stderr, "[warn] unknown flag ignored: %s\n", a);
    }
    return c;
}

// A raw field of n values in C order, float64 or float32 (read_raw_field_to_double,
// main_cuda.cu:2764-2799: the size must match exactly), widened to double.
bool read_raw(const std::string &path, size_t n, std::vector<double> *out, bool f32 = false) {
    const size_t esz = f32 ? sizeof(float) : sizeof(double);
    FILE *f = fopen(path.c_str(), "rb");
    if (!f) { fprintf(stderr, "[fatal] cannot open raw field %s\n", path.c_str()); return false; }
    fseek(f, 0, SEEK_END);
    const long sz = ftell(f);
    fseek(f, 0, SEEK_SET);
    if (sz != (long)(n * esz)) {
        fprintf(stderr, "[fatal] raw field %s has %ld bytes, expected %zu (%s x %zu)\n", path.c_str(), sz, n * esz,
                f32 ? "float32" : "float64", n);
        fclose(f);
        return false;
    }
    out->resize(n);
    size_t got;
    if (f32) {
        std::vector<float> tmp(n);
        got = fread(tmp.data(), sizeof(float), n, f);
        for (size_t i = 0; i < n; ++i) (*out)[i] = tmp[i];
    } else {
        got = fread(out->data(), sizeof(double), n, f);
    }
    fclose(f);
    if (got != n) { fprintf(stderr, "[fatal] short read of %s\n", path.c_str()); return false; }
    return true;
}

std::string slurp(const std::string &path) {
    std::string s;
    FILE *f = fopen(path.c_str(), "rb");
    if (!f) return s;
    char buf[4096];
    size_t k;
    while ((k = fread(buf, 1, sizeof(buf), f)) > 0) s.append(buf, k);
    fclose(f);
    return s;
}

// number after "key": in a flat JSON text (init_meta.json); false if absent
bool json_number(const std::string &txt, const char *key, double *v) {
    const std::string k = std::string("\"") + key + "\"";
    size_t p = txt.find(k);
    if (p == std::string::npos) return false;
    p = txt.find(':', p + k.size());
    if (p == std::string::npos) return false;
    const char *s = txt.c_str() + p + 1;
    char *e = nullptr;
    const double x = strtod(s, &e);
    if (e == s) return false;
    *v = x;
    return true;
}

// string after "key": in a flat JSON text; false if absent
bool json_string(const std::string &txt, const char *key, std::string *v) {
    const std::string k = std::string("\"") + key + "\"";
    size_t p = txt.find(k);
    if (p == std::string::npos) return false;
    p = txt.find(':', p + k.size());
    if (p == std::string::npos) return false;
    const size_t q0 = txt.find('"', p + 1);
    if (q0 == std::string::npos) return false;
    const size_t q1 = txt.find('"', q0 + 1);
    if (q1 == std::string::npos) return false;
    *v = txt.substr(q0 + 1, q1 - q0 - 1);
    return true;
}

// ASCII VTK scalar field (read_vtk_ascii_to_host, io_vtk_cuda.h:131-200):
// DIMENSIONS must match (a 2D x-z file has Ny = 1 for a run with Ny = 2),
// values follow LOOKUP_TABLE with x fastest, then y, then z
bool read_vtk_field(const std::string &path, int Nx, int Ny, int Nz, std::vector<double> *out) {
    FILE *f = fopen(path.c_str(), "r");
    if (!f) { fprintf(stderr, "ERROR: Cannot open VTK file %s for reading\n", path.c_str()); return false; }
    char line[4096];
    int vx = -1, vy = -1, vz = -1;
    bool dims = false, lookup = false;
    while (fgets(line, sizeof(line), f)) {
        if (!dims && !strncmp(line, "DIMENSIONS", 10)) { dims = sscanf(line, "DIMENSIONS %d %d %d", &vx, &vy, &vz) == 3; continue; }
        if (!strncmp(line, "LOOKUP_TABLE", 12)) { lookup = true; break; }
    }
    const bool two_d = vy == 1 && Ny == 2;
    if (!dims || !lookup || vx != Nx || vz != Nz || !(vy == Ny || two_d)) {
        fprintf(stderr, "ERROR: VTK grid mismatch or bad header in %s: file=%dx%dx%d expected=%dx%dx%d\n",
                path.c_str(), vx, vy, vz, Nx, Ny, Nz);
        fclose(f);
        return false;
    }
    out->assign((size_t)Nx * Ny * Nz, 0.0);
    const int ny_in = two_d ? 1 : Ny;
    for (int k = 0; k < Nz; ++k)
        for (int j = 0; j < ny_in; ++j)
            for (int i = 0; i < Nx; ++i) {
                double v;
                if (fscanf(f, "%lf", &v) != 1) {
                    fprintf(stderr, "ERROR: Unexpected EOF while reading VTK data from %s\n", path.c_str());
                    fclose(f);
                    return false;
                }
                for (int jj = j; jj < (two_d ? Ny : j + 1); ++jj) (*out)[((size_t)i * Ny + jj) * Nz + k] = v;
            }
    fclose(f);
    return true;
}

double h_of(double p);
double clamp_eps_h(double x, double e) { return x < e ? e : (x > 1.0 - e ? 1.0 - e : x); }

// volume fraction of the legacy seed target (compute_effective_vf_target,
// main_cuda.cu:2459-2490; ellipsoid axes normalised to the sphere's volume)
double effective_vf_target(const pfgb_params &P) {
    const double vf = std::fmin(0.999, std::fmax(1e-6, P.ic_vf_target_phi));
    if (!(P.ic_phi_seed_radius > 0.0)) return vf;
    const int ns = P.ic_phi_num_seeds > 0 ? P.ic_phi_num_seeds : 1;
    const double R = P.ic_phi_seed_radius, Lx = P.Nx * P.dx, Ly = P.Ny * P.dy, Lz = P.Nz * P.dz;
    double t = vf;
    if (P.Ny > 2) { if (Lx * Ly * Lz > 0.0) t = ns * (4.0 * M_PI / 3.0) * R * R * R / (Lx * Ly * Lz); }
    else if (Lx * Lz > 0.0) t = ns * M_PI * R * R / (Lx * Lz);
    return std::fmin(0.999, std::fmax(1e-6, t));
}

// composition rebuilt from phi by the diffuse-interface lever rule
// (rebuild_full_model_composition_from_phi, main_cuda.cu:2521-2600)
void rebuild_composition(const pfgb_params &P, std::vector<double> &phi, std::vector<double> *xB) {
    const size_t N = phi.size();
    double sh = 0.0, sh2 = 0.0;
    for (size_t i = 0; i < N; ++i) {
        phi[i] = std::fmin(1.0, std::fmax(0.0, phi[i]));
        const double h = h_of(phi[i]);
        sh += h;
        sh2 += h * h;
    }
    const double mh = sh / (double)N, mh2 = sh2 / (double)N, xeq = P.xB_eq_matrix, vf = effective_vf_target(P);
    const double target = P.v_B * vf + (1.0 - vf) * xeq;
    const double A = 1.0 - 2.0 * mh + mh2, B = mh - mh2, C = P.v_B * mh;
    double xout;
    if (P.ic_23d_xB_out > 0.0) xout = P.ic_23d_xB_out;
    else if (std::fabs(A) < 1e-12) xout = ((vf - mh) * P.v_B + (1.0 - vf) * xeq) / std::fmax(1.0 - mh, 1e-12);
    else xout = (target - B * xeq - C) / A;
    xout = clamp_eps_h(xout, P.xB_eps);
    xB->resize(N);
    for (size_t i = 0; i < N; ++i) {
        const double h = h_of(phi[i]);
        (*xB)[i] = clamp_eps_h((1.0 - h) * xout + h * xeq, P.xB_eps);
    }
}

// continue_dyn_<n+1> / continue_min_<n+1>, n the largest index of that
// prefix in the source path (derive_next_continue_case_tag, main_cuda.cu:2492-2520)
std::string next_continue_tag(const std::string &path, bool minimize) {
    const std::string prefix = minimize ? "continue_min_" : "continue_dyn_";
    int mx = 0;
    for (size_t p = path.find(prefix); p != std::string::npos; p = path.find(prefix, p + 1)) {
        size_t q = p + prefix.size();
        if (q < path.size() && isdigit((unsigned char)path[q])) {
            int v = 0;
            while (q < path.size() && isdigit((unsigned char)path[q])) v = v * 10 + (path[q++] - '0');
            mx = std::max(mx, v);
        }
    }
    return prefix + std::to_string(mx + 1);
}

std::string dir_of(const std::string &p) {
    const size_t s = p.rfind('/');
    return s == std::string::npos ? std::string() : p.substr(0, s);
}
std::string base_of(const std::string &p) {
    const size_t s = p.rfind('/');
    return s == std::string::npos ? p : p.substr(s + 1);
}

// last step, t_code, t_real of an existing vf CSV / last iteration of an
// energy CSV (read_last_vf_csv_state / read_last_energy_iter, main_cuda.cu:311-352)
bool last_csv_row(const std::string &path, int *step, double *t, double *tr) {
    FILE *f = fopen(path.c_str(), "r");
    if (!f) return false;
    char line[4096];
    bool found = false;
    while (fgets(line, sizeof(line), f)) {
        if (!isdigit((unsigned char)line[0]) && line[0] != '-') continue;
        int a;
        double b = 0.0, d = 0.0;
        const int n = sscanf(line, "%d,%lf,%lf", &a, &b, &d);
        if ((tr && n == 3) || (!tr && n >= 1)) {
            found = true;
            *step = a;
            if (t) *t = b;
            if (tr) *tr = d;
        }
    }
    fclose(f);
    return found;
}

// a key of the parameter file that the library's parameter struct does not
// carry (used for output naming only)
double param_file_value(const std::string &txt, const char *key, double dflt) {
    size_t p = 0;
    while (p < txt.size()) {
        size_t e = txt.find('\n', p);
        if (e == std::string::npos) e = txt.size();
        std::string line = txt.substr(p, e - p);
        p = e + 1;
        const size_t hash = line.find('#');
        if (hash != std::string::npos) line.resize(hash);
        const size_t eq = line.find('=');
        if (eq == std::string::npos) continue;
        std::string k = line.substr(0, eq), v = line.substr(eq + 1);
        auto trim = [](std::string &s) {
            while (!s.empty() && isspace((unsigned char)s.back())) s.pop_back();
            size_t b = 0;
            while (b < s.size() && isspace((unsigned char)s[b])) ++b;
            s.erase(0, b);
        };
        trim(k); trim(v);
        double x;
        if (k == key && to_double(v.c_str(), &x)) return x;
    }
    return dflt;
}

bool copy_file(const std::string &from, const std::string &to) {
    const std::string s = slurp(from);
    FILE *f = fopen(to.c_str(), "wb");
    if (!f) return false;
    fwrite(s.data(), 1, s.size(), f);
    fclose(f);
    return true;
}

// ASCII STRUCTURED_POINTS, z outermost, x innermost, %.5f (io_vtk_cuda.h:80-128)
bool write_vtk(const std::string &vtk_path, const char *name, const std::vector<double> &v, int Nx, int Ny, int Nz,
               int step = -1) {
    const char *sup = getenv("CUDA_STO_SUPPRESS_VTK_OUTPUT");   // io_vtk_cuda.h:17-45
    if (sup && strcmp(sup, "1") == 0) {
        printf("VTK_OUTPUT_SUPPRESSED field=%s step=%d path=%s\n", name, step, vtk_path.c_str());
        return true;
    }
    std::string path = vtk_path;
    if (g_out_fmt == OutFmt::Raw && path.size() > 4 && path.compare(path.size() - 4, 4, ".vtk") == 0)
        path = path.substr(0, path.size() - 4) + ".raw";
    FILE *fo = fopen(path.c_str(), g_out_fmt == OutFmt::VtkAscii ? "w" : "wb");
    if (!fo) { fprintf(stderr, "ERROR: Cannot create file %s\n", path.c_str()); return false; }
    bool ok = true;
    if (g_out_fmt == OutFmt::Raw) {
        ok = fwrite(v.data(), sizeof(double), v.size(), fo) == v.size();
        return (fclose(fo) == 0) && ok;
    }
    const int ny_out = Ny == 2 ? 1 : Ny;
    const bool bin = g_out_fmt == OutFmt::VtkBinary;
    fprintf(fo, "# vtk DataFile Version 3.0\nPhase Field Simulation\n%s\nDATASET STRUCTURED_POINTS\n",
            bin ? "BINARY" : "ASCII");
    fprintf(fo, "DIMENSIONS %d %d %d\nASPECT_RATIO 1 1 1\nORIGIN 0 0 0\nPOINT_DATA %d\n", Nx, ny_out, Nz,
            Nx * ny_out * Nz);
    fprintf(fo, "SCALARS %s double 1\nLOOKUP_TABLE default\n", name);
    std::string line;
    char tmp[64];
    std::vector<unsigned char> row((size_t)Nx * 8);
    for (int k = 0; k < Nz; ++k)
        for (int j = 0; j < ny_out; ++j) {
            if (bin) {
                for (int i = 0; i < Nx; ++i) {   // big-endian, as legacy VTK binary requires
                    uint64_t u;
                    const double d = v[((size_t)i * Ny + j) * Nz + k];
                    memcpy(&u, &d, 8);
                    for (int b = 0; b < 8; ++b) row[(size_t)i * 8 + b] = (unsigned char)(u >> (56 - 8 * b));
                }
                ok = ok && fwrite(row.data(), 1, row.size(), fo) == row.size();
                continue;
            }
            line.clear();
            for (int i = 0; i < Nx; ++i) {
                const int n = snprintf(tmp, sizeof(tmp), "%.5f ", v[((size_t)i * Ny + j) * Nz + k]);
                line.append(tmp, n);
            }
            ok = ok && fwrite(line.data(), 1, line.size(), fo) == line.size();
        }
    fprintf(fo, "\n");
    return (fclose(fo) == 0) && ok;
}

double h_of(double p) { return p * p * p * (6.0 * p * p - 15.0 * p + 10.0); }

std::string now_str() {
    char b[64];
    time_t t = time(nullptr);
    struct tm *lt = localtime(&t);
    if (!lt || !strftime(b, sizeof(b), "%Y-%m-%d %H:%M:%S", lt)) return "unknown";
    return b;
}

int fail(pfgb_status s, const char *where) {
    fprintf(stderr, "[fatal] %s: %s (%s)\n", where, pfgb_status_string(s), pfgb_last_error(nullptr));
    return s == PFGB_ERR_CUDA || s == PFGB_ERR_NOMEM ? 1 : 2;
}

}  // namespace

int main(int argc, char **argv) {
    Cli c = parse(argc, argv);
    if (c.param_file.empty()) {
        fprintf(stderr, "[fatal] --pf-param-file <path> is required (complete physical PF inputs).\n");
        return 2;
    }
    // dynamics-continue is the dynamics run under another name
    // (main_cuda.cu:22752-22763); its raw-field / checkpoint inputs are the
    // ordinary ones
    if (c.mode == "dynamics-continue") c.mode = "dynamics";
    if (c.mode == "minimize-continue") { c.mode = "minimize"; c.cont = true; }
    if (c.mode != "dynamics" && c.mode != "minimize") {
        fprintf(stderr, "[fatal] --mode=%s is not available in this program (dynamics, dynamics-continue, minimize)\n",
                c.mode.c_str());
        return 2;
    }
    const bool minimize = c.mode == "minimize";
    pfgb_params P;
    pfgb_params_default(&P);
    if (c.pos_Nx > 0) P.Nx = c.pos_Nx;
    if (c.pos_Ny > 0) P.Ny = c.pos_Ny;
    if (c.pos_Nz > 0) P.Nz = c.pos_Nz;
    if (std::isfinite(c.pos_dt)) P.dt = c.pos_dt;
    if (c.pos_elastic >= 0) P.elastic_enabled = c.pos_elastic ? 1 : 0;
    char err[512] = {0};
    pfgb_status st = pfgb_params_load_file(&P, c.param_file.c_str(), err, sizeof(err));
    if (st != PFGB_OK) {
        fprintf(stderr, "[fatal] %s\n", err);
        return 2;
    }
    // the parameter file does not set the grid: positional values stand
    if (c.pos_Nx > 0) P.Nx = c.pos_Nx;
    if (c.pos_Ny > 0) P.Ny = c.pos_Ny;
    if (c.pos_Nz > 0) P.Nz = c.pos_Nz;
    // the positional elastic switch is a default the parameter file may
    // override (it is set before the file is read, main_cuda.cu:22534-22540);
    // the --elastic flag is read after it and wins
    if (c.elastic >= 0) P.elastic_enabled = c.elastic ? 1 : 0;
    if (std::isfinite(c.temperature_C)) P.temperature_C = c.temperature_C;
    if (!c.zero_mode.empty()) {
        if (c.zero_mode == "PF_CONSERVED_Y_ZERO_MODE_V1") P.zero_mode_enabled = 1;
        else if (c.zero_mode == "OFF") P.zero_mode_enabled = 0;
        else bad("--pf-zero-mode", c.zero_mode.c_str());
    }
    if (std::isfinite(c.zm_tol)) P.zero_mode_tolerance_relative = c.zm_tol;
    if (c.zm_maxit > 0) P.zero_mode_max_iterations = c.zm_maxit;
    if (c.prev_level) P.enable_Y_rhs_previous_time_level = 1;
    if (c.no_gamma) P.disable_Y_rhs_gamma_term = 1;
    if (std::isfinite(c.h_scale)) P.Y_rhs_term_h_scale = c.h_scale;
    P.precision = c.precision;
    if (minimize) {
        P.mode = PFGB_MODE_MINIMIZE;
        P.minimize_dt = P.dt;   // the parameter file's dt unless --minimize-dt is given
        if (c.min_full) P.minimize_full_model = 1;
        if (c.min_max_iter > 0) P.minimize_max_iter = c.min_max_iter;
        if (std::isfinite(c.min_dt)) P.minimize_dt = c.min_dt;
        if (std::isfinite(c.V0)) P.minimize_V0 = c.V0;
        if (std::isfinite(c.eta_lambda)) P.eta_lambda_vol = c.eta_lambda;
        if (std::isfinite(c.thr_dphi)) P.minimize_rms_dphi_threshold = c.thr_dphi;
        if (std::isfinite(c.thr_dY)) P.minimize_rms_dY_threshold = c.thr_dY;
        if (std::isfinite(c.thr_res)) P.minimize_rms_res_threshold = c.thr_res;
        if (std::isfinite(c.thr_vol)) P.minimize_vol_err_rel_threshold = c.thr_vol;
        if (std::isfinite(c.thr_E)) P.minimize_energy_diff_rel_threshold = c.thr_E;
        if (c.min_conv_steps > 0) P.minimize_convergence_steps = c.min_conv_steps;
        if (c.min_post_iters >= 0) P.minimize_post_projection_iters = c.min_post_iters;
        if (std::isfinite(c.min_pt)) P.minimize_min_pseudo_time = c.min_pt;
        if (std::isfinite(c.xB_max_safe)) P.minimize_xB_max_safe = c.xB_max_safe;
        c.nsteps = P.minimize_max_iter;   // main_cuda.cu:24432-24435
        P.dt = P.minimize_dt;
    }
    if (std::isfinite(c.radius)) P.ic_phi_seed_radius = c.radius;
    for (const auto &kv : c.param_sets)
        if (pfgb_params_set(&P, kv.first.c_str(), kv.second.c_str()) != PFGB_OK) bad(kv.first.c_str(), kv.second.c_str());
    if (c.tilt_given && (P.init_tilt_theta_deg != 0.0 || P.init_tilt_phi_deg != 0.0)) P.init_use_rotation = 1;
    // the zero mode is a dynamics-only two-phase mode (main_cuda.cu:24662-24690);
    // the library also runs it with gp_zone, the drop-in driver refuses it
    if (P.zero_mode_enabled && (minimize || P.model_mode == PFGB_MODEL_GP_ZONE)) {
        fprintf(stderr, "[fatal] PF_CONSERVED_Y_ZERO_MODE_V1 is a dynamics-only PF mode and requires every GP, "
                        "RSMD, scheduled-source, and bridge path OFF\n");
        return 2;
    }
    if (std::isfinite(c.radius_nm)) {   // main_cuda.cu:25288-25310: physical radius -> code units
        const double dxp = P.ic_phi_iface_w > 1e-30 ? P.lambda_sm_m / (2.0 * P.ic_phi_iface_w) : P.dx * 1e-9;
        const double u2m = std::fabs(P.dx) > 1e-30 ? dxp / P.dx : 1e-9;
        P.ic_phi_seed_radius = c.radius_nm * 1e-9 / u2m;
    }
    if (c.nsteps < 0 || c.out_every <= 0 || c.csv_out_every <= 0) {
        fprintf(stderr, "[fatal] nsteps >= 0, out_every > 0 and csv_out_every > 0 are required\n");
        return 2;
    }
    if (c.warm_source >= 0) P.elastic_warm_start_source = c.warm_source;
    else if (!c.warm_model.empty()) P.elastic_warm_start_source = 1;
    if ((P.elastic_warm_start_source == 1 || P.elastic_warm_start_source == 2) && c.warm_model.empty()) {
        fprintf(stderr, "[fatal] --elastic-warm-start-source %d needs --elastic-warm-start-model\n",
                P.elastic_warm_start_source);
        return 2;
    }
    // checkpoint contract (main_cuda.cu:22760-22790)
    const bool restarting = !c.restart_from.empty();
    if (c.ckpt_every < 0) { fprintf(stderr, "[fatal] --pf-checkpoint-every must be >= 0\n"); return 2; }
    if ((c.ckpt_every > 0 || restarting) && !P.zero_mode_enabled) {
        fprintf(stderr, "[fatal] PF checkpoint/restart provenance is available only with "
                        "PF_CONSERVED_Y_ZERO_MODE_V1\n");
        return 2;
    }
    if (c.ckpt_every > 0 && c.ckpt_path.empty()) {
        fprintf(stderr, "[fatal] --pf-checkpoint-path is required when periodic checkpointing is enabled\n");
        return 2;
    }
    if ((c.ckpt_every > 0 || restarting) && minimize) {
        fprintf(stderr, "[fatal] checkpoints are written and read by dynamics runs only\n");
        return 2;
    }
    if ((st = pfgb_params_finalize(&P)) != PFGB_OK) return fail(st, "pfgb_params_finalize");

    // ---- initial fields ---------------------------------------------------
    const size_t N = (size_t)P.Nx * P.Ny * P.Nz;
    std::vector<double> phi, xB, eta, dYdt;
    // VTK continuation (main_cuda.cu:24752-24772, 27194-27207)
    if (c.cont) {
        if (c.cont_phi.empty()) {
            fprintf(stderr, "[fatal] continuation needs --continue-phi-vtk <path>\n");
            return 2;
        }
        if (!c.init_mode.empty()) {
            fprintf(stderr, "[fatal] --init-mode raw_fields cannot be combined with --continue-phi-vtk/--continue-xB-vtk.\n");
            return 2;
        }
        if (P.zero_mode_enabled || restarting) {
            fprintf(stderr, "[fatal] zero-mode restart cannot be mixed with VTK continuation; use --pf-restart-from "
                            "for exact state restoration\n");
            return 2;
        }
        printf("[continue-param] explicit --pf-param-file takes precedence over stored PF params next to %s\n",
               c.cont_phi.c_str());
    }
    const bool seeded = !restarting && !c.cont && c.init_mode.empty();
    if (c.cont) {
        if (!read_vtk_field(c.cont_phi, P.Nx, P.Ny, P.Nz, &phi)) return 2;
        if (!minimize || P.minimize_full_model) {
            struct stat sb;
            if (!c.cont_xB.empty() && stat(c.cont_xB.c_str(), &sb) == 0) {
                if (!read_vtk_field(c.cont_xB, P.Nx, P.Ny, P.Nz, &xB)) return 2;
            } else {
                if (!c.cont_xB.empty())
                    fprintf(stderr, "[warn] continuation xB VTK missing or unreadable, xB/Y rebuilt from phi: %s\n",
                            c.cont_xB.c_str());
                rebuild_composition(P, phi, &xB);
            }
        } else {
            xB.assign(N, 0.0);   // phi-only minimize carries no composition
        }
        // clamps only (no xB_max_safe cap): phi to [0, 1], xB to [eps, 1 - eps]
        st = pfgb_prepare_raw_fields(&P, NAN, phi.data(), xB.data(), nullptr, nullptr, N);
        if (st != PFGB_OK) return fail(st, "pfgb_prepare_raw_fields");
    } else if (restarting || seeded) {
        // the fields come from the checkpoint (main_cuda.cu:27340-27380) or
        // from the seeded initialiser on the device (main_cuda.cu:15157-15430)
    } else if (c.init_mode != "raw_fields") {
        fprintf(stderr, "[fatal] unknown --init-mode %s (raw_fields, or none for the seeded initialiser)\n",
                c.init_mode.c_str());
        return 2;
    } else if (c.init_phi.empty() || c.init_xB.empty()) {
        fprintf(stderr, "[fatal] raw_fields needs --init-phi-raw and --init-xB-raw\n");
        return 2;
    }
    if (!restarting && !seeded && !c.cont && minimize && !P.minimize_full_model) {
        fprintf(stderr, "[fatal] --init-mode raw_fields requires dynamics mode or full-model minimize "
                        "(--mode=minimize --minimize-full-model).\n");
        return 2;
    }
    if (!restarting && !seeded && !c.cont) {
        // init_meta.json (load_raw_init_meta, main_cuda.cu:2733-2762): the
        // grid must match, order must be C, dtype is float32 (the default)
        // or float64, and xB_max_safe caps xB (the minimize monitor cap when
        // absent).  Without --init-meta the fields are read as float64.
        double xB_max_safe = P.minimize_xB_max_safe;
        bool f32 = false;
        if (!c.init_meta.empty()) {
            const std::string meta = slurp(c.init_meta);
            if (meta.empty()) { fprintf(stderr, "[fatal] cannot read raw init meta: %s\n", c.init_meta.c_str()); return 2; }
            double v;
            if (json_number(meta, "xB_max_safe", &v)) xB_max_safe = v;
            const char *dims[3] = {"Nx", "Ny", "Nz"};
            const int have[3] = {P.Nx, P.Ny, P.Nz};
            for (int a = 0; a < 3; ++a)
                if (json_number(meta, dims[a], &v) && (int)v != have[a]) {
                    fprintf(stderr, "[fatal] init_meta %s=%d does not match the grid (%d)\n", dims[a], (int)v, have[a]);
                    return 2;
                }
            std::string dtype = "float32", order = "C";
            json_string(meta, "dtype", &dtype);
            json_string(meta, "order", &order);
            if (order != "C") {
                fprintf(stderr, "[fatal] raw init order mismatch: meta order='%s', only C is supported\n", order.c_str());
                return 2;
            }
            if (dtype != "float32" && dtype != "float64") {
                fprintf(stderr, "[fatal] unsupported raw dtype '%s'; use float32 or float64\n", dtype.c_str());
                return 2;
            }
            f32 = dtype == "float32";
        }
        if (!read_raw(c.init_phi, N, &phi, f32) || !read_raw(c.init_xB, N, &xB, f32)) return 2;
        if (!c.init_eta.empty() && !read_raw(c.init_eta, N, &eta, f32)) return 2;
        if (!c.init_dYdt.empty() && !read_raw(c.init_dYdt, N, &dYdt, f32)) return 2;
        st = pfgb_prepare_raw_fields(&P, xB_max_safe, phi.data(), xB.data(), eta.empty() ? nullptr : eta.data(),
                                     dYdt.empty() ? nullptr : dYdt.data(), N);
        if (st != PFGB_OK) return fail(st, "pfgb_prepare_raw_fields");
    }

    // ---- output layout ----------------------------------------------------
    const std::string ptxt = slurp(c.param_file);
    const double xB_out = param_file_value(ptxt, "ic_23d_xB_out", param_file_value(ptxt, "xB_alpha_initial", 0.03));
    const char *root_env = getenv("CUDA_STO_RESULTS_ROOT");
    const std::string root = (root_env && root_env[0]) ? root_env : "Results";
    const double dx_phys = P.ic_phi_iface_w > 1e-30 ? P.lambda_sm_m / (2.0 * P.ic_phi_iface_w) : P.dx * 1e-9;
    const double unit_to_m = std::fabs(P.dx) > 1e-30 ? dx_phys / P.dx : 1e-9;
    const double unit_to_nm = unit_to_m * 1e9;
    char name[512];
    if (minimize)   // named with the physical seed radius (main_cuda.cu:25386-25396)
        snprintf(name, sizeof(name), "%s_T%.0f_cuda_%dx%dx%d_dt%.3g_steps%d_r%.3fnm_xB%.3f",
                 P.elastic_enabled ? "chel" : "ch", P.temperature_C, P.Nx, P.Ny, P.Nz, P.dt, c.nsteps,
                 P.ic_phi_seed_radius * unit_to_nm, xB_out);
    else
        snprintf(name, sizeof(name), "%s_T%.0f_cuda_%dx%dx%d_dt%.3g_steps%d_xB%.3f", P.elastic_enabled ? "chel" : "ch",
                 P.temperature_C, P.Nx, P.Ny, P.Nz, P.dt, c.nsteps, xB_out);
    mkdir(root.c_str(), 0755);
    std::string out_dir = root + "/" + name, tag = c.case_tag, csv_tag;
    if (c.cont) {
        // the source run's root (the phi VTK's case directory's parent): kept,
        // or re-rooted under CUDA_STO_RESULTS_ROOT by its base name
        // (main_cuda.cu:25363-25385); a new case directory continue_*_<n>
        const std::string src_case = dir_of(c.cont_phi), src_root = dir_of(src_case);
        if (root_env && root_env[0] && !base_of(src_root).empty()) out_dir = root + "/" + base_of(src_root);
        else out_dir = !src_root.empty() ? src_root : root;
        if (tag.empty()) tag = next_continue_tag(c.cont_phi, minimize);
        csv_tag = !src_case.empty() ? base_of(src_case) : tag;
    }
    mkdir(out_dir.c_str(), 0755);
    if (!minimize && !c.cont) copy_file(c.param_file, out_dir + "/pf_input.params");   // main_cuda.cu:25408-25416
    if (tag.empty() && seeded) {   // main_cuda.cu:25425-25436
        char t[256];
        snprintf(t, sizeof(t), "case_test%d_%s_th%.0f_ph%.0f_noise%.0e", -1,
                 P.init_shape_mode == 0 ? "sphere" : P.init_shape_mode == 1 ? "ellipsoid" : "legacy",
                 P.init_tilt_theta_deg, P.init_tilt_phi_deg, P.init_phi_noise_amp);
        tag = t;
    }
    if (tag.empty()) tag = "raw_fields_relax";
    if (csv_tag.empty()) csv_tag = tag;
    const std::string case_dir = out_dir + "/" + tag;
    mkdir(case_dir.c_str(), 0755);
    copy_file(c.param_file, case_dir + "/pf_input.params");
    const bool gp = P.model_mode == PFGB_MODEL_GP_ZONE;
    // gp_storage_coupling_enabled (main_cuda.cu:16767-16772): the outputs carry
    // xBtot_gp = h_alpha x + h_GP x_GP + h_beta (xBtot_output_stem,
    // xBtot_vtk_field_name, main_cuda.cu:16774-16780)
    const bool gpc = gp && (P.enable_legacy_gp_storage_coupling || !P.gp_barrier_only_mode);
    const std::string xbt_stem = gpc ? "/xBtot_gp" : "/xBtot";
    const char *xbt_name = gpc ? "xBtot_gp" : "xB_tot";
    printf("output_dir=%s\ncase_output_dir=%s\n", out_dir.c_str(), case_dir.c_str());

    // ---- solver -----------------------------------------------------------
    struct ModelHolder {   // released after the context (declared first)
        pfgb_fno *m = nullptr;
        ~ModelHolder() { if (m) pfgb_fno_destroy(m); }
    } model;
    pfgb_ctx *ctx = nullptr;
    if ((st = pfgb_create(&P, c.device, &ctx)) != PFGB_OK) return fail(st, "pfgb_create");
    if (!c.warm_model.empty()) {
        if ((st = pfgb_fno_load(c.warm_model.c_str(), P.Nx, P.Ny, P.Nz, c.device, &model.m)) != PFGB_OK ||
            (st = pfgb_set_warm_start_model(ctx, model.m)) != PFGB_OK) {
            pfgb_destroy(ctx);
            return fail(st, "--elastic-warm-start-model");
        }
    }
    int first_step = 1;
    if (restarting) {
        st = pfgb_checkpoint_restore(ctx, c.restart_from.c_str(), c.isc.c_str(), c.fsha.c_str(), c.psha.c_str());
        if (st != PFGB_OK) { pfgb_destroy(ctx); return fail(st, "PF zero-mode restart rejected"); }
        pfgb_step_stats s0;
        if ((st = pfgb_step(ctx, 0, &s0)) != PFGB_OK) { pfgb_destroy(ctx); return fail(st, "pfgb_step"); }
        if (s0.step >= c.nsteps) {
            fprintf(stderr, "[fatal] restart accepted_step=%d must be less than requested final nsteps=%d\n",
                    s0.step, c.nsteps);
            pfgb_destroy(ctx);
            return 2;
        }
        first_step = s0.step + 1;
        printf("PF_ZERO_MODE_RESTART checkpoint=%s accepted_step=%d\n", c.restart_from.c_str(), s0.step);
    } else if (seeded && !c.cont) {
        if ((st = pfgb_init_fields(ctx)) != PFGB_OK) { pfgb_destroy(ctx); return fail(st, "pfgb_init_fields"); }
        if (minimize && !P.minimize_full_model) {
            // phi-only minimize starts from the seeded phi with no composition
            // (initialize_phi_only_cuda and the zeroed xB / Y, main_cuda.cu:27208-27217)
            std::vector<double> p0(N), x0(N, 0.0);
            if ((st = pfgb_read_fields(ctx, p0.data(), nullptr, nullptr, nullptr, nullptr)) != PFGB_OK ||
                (st = pfgb_load_fields(ctx, p0.data(), x0.data(), nullptr, nullptr)) != PFGB_OK) {
                pfgb_destroy(ctx);
                return fail(st, "phi-only minimize initial fields");
            }
        }
    } else {
        st = pfgb_load_fields(ctx, phi.data(), xB.data(), eta.empty() ? nullptr : eta.data(),
                              dYdt.empty() ? nullptr : dYdt.data());
        if (st != PFGB_OK) { pfgb_destroy(ctx); return fail(st, "pfgb_load_fields"); }
    }

    std::vector<double> f_phi(N), f_xB(N), f_eta(N), f_xBtot(N);
    auto read_state = [&]() -> pfgb_status {
        return pfgb_read_fields(ctx, f_phi.data(), f_xB.data(), nullptr, gp ? f_eta.data() : nullptr, nullptr);
    };
    auto vtk_set = [&](const char *suffix, int step) -> bool {
        // launch_compute_model_xBtot_kernel (main_cuda.cu:19855-19866)
        for (size_t i = 0; i < N; ++i) {
            const double h = h_of(f_phi[i]);
            if (gpc) {
                const double he = h_of(f_eta[i]);
                f_xBtot[i] = (1.0 - h) * (1.0 - he) * f_xB[i] + (1.0 - h) * he * P.gp_xB_fixed + h;
            } else {
                f_xBtot[i] = (1.0 - h) * f_xB[i] + h * P.v_B;
            }
        }
        // the fields of one output set are written in parallel
        struct Job { std::string path; const char *name; const std::vector<double> *v; bool ok; };
        std::vector<Job> jobs = {{case_dir + xbt_stem + suffix + ".vtk", xbt_name, &f_xBtot, false},
                                 {case_dir + "/xB" + suffix + ".vtk", "xB", &f_xB, false},
                                 {case_dir + "/phi" + suffix + ".vtk", "phi", &f_phi, false}};
        if (gp) jobs.push_back({case_dir + "/eta" + suffix + ".vtk", "eta", &f_eta, false});
        std::vector<std::thread> th;
        for (Job &j : jobs)
            th.emplace_back([&j, &P, step]() { j.ok = write_vtk(j.path, j.name, *j.v, P.Nx, P.Ny, P.Nz, step); });
        for (std::thread &t : th) t.join();
        bool ok = true;
        for (const Job &j : jobs) ok = ok && j.ok;
        return ok;
    };

    // vf CSV (dynamics and full-model minimize, main_cuda.cu:25571-25590); a
    // continuation appends to an existing one, its rows offset by the last row
    int csv_step_off = 0;
    double csv_t_off = 0.0, csv_tr_off = 0.0;
    const bool want_csv = !minimize || P.minimize_full_model;
    const std::string csv_path = case_dir + "/vf_precip_vs_time_" + csv_tag + ".csv";
    const bool csv_append = c.cont && last_csv_row(csv_path, &csv_step_off, &csv_t_off, &csv_tr_off);
    FILE *csv = want_csv ? fopen(csv_path.c_str(), csv_append ? "a" : "w") : nullptr;
    FILE *etrace = nullptr, *ztrace = nullptr;
    const bool accel = P.elastic_enabled && (P.elastic_warm_start_enabled || P.elastic_residual_control_enabled);
    if (accel) {
        etrace = fopen((case_dir + "/elastic_solver_trace.csv").c_str(), "w");
        if (etrace)
            fprintf(etrace, "step,warm_start_used,iterations,relative_residual,converged,hard_cap,tolerance,"
                            "solver_wall_s,source_field_step\n");
    }
    if (P.zero_mode_enabled) {
        ztrace = fopen((case_dir + "/pf_zero_mode_trace.csv").c_str(), "w");
        if (ztrace)
            fprintf(ztrace, "step,target_mass_code,lambda,residual_code,derivative_code,iterations,newton_steps,"
                            "bisection_steps,Y_star_min,Y_star_max,lambda_lower,lambda_upper,"
                            "accepted_zero_mode_steps\n");
    }
    if ((want_csv && !csv) || (accel && !etrace) || (P.zero_mode_enabled && !ztrace)) {
        fprintf(stderr, "[fatal] cannot open the CSV outputs under %s\n", case_dir.c_str());
        pfgb_destroy(ctx);
        return 2;
    }
    if (csv && !csv_append) fprintf(csv, "step,t_code,t_real_s,vf_precip,R_avg\n");
    FILE *efp = nullptr;
    int energy_off = 0;
    if (minimize) {   // energy_minimize_T%.0f_r%.2f_xB%.3f_<tag>.csv (main_cuda.cu:27436-27467)
        char en[512];
        snprintf(en, sizeof(en), "/energy_minimize_T%.0f_r%.2f_xB%.3f_%s.csv", P.temperature_C, P.ic_phi_seed_radius,
                 xB_out, csv_tag.c_str());
        const bool e_append = c.cont && last_csv_row(case_dir + en, &energy_off, nullptr, nullptr);
        efp = fopen((case_dir + en).c_str(), e_append ? "a" : "w");
        if (!efp) { fprintf(stderr, "[fatal] cannot open %s%s\n", case_dir.c_str(), en); pfgb_destroy(ctx); return 2; }
        if (!e_append)
            fprintf(efp, "iter,dt,mean_h,V0,lambda,F_surf_hat,F_el_hat,F_chem_excess_hat,F_total_excess_hat,"
                         "F_chem_CNT_hat,F_total_CNT_hat,total_interface_sum,total_el_core_sum,"
                         "rms_res,rms_dphi,rms_dY,rel_dF,vol_err_rel,mass_target_code,mass_current_code,mass_err_rel,"
                         "mass_lambda,post_proj_iters_used\n");
    }

    const char *dim = P.Ny == 2 ? "[2D]" : "[3D]";
    auto csv_row = [&](int step, double vf_override) -> pfgb_status {
        pfgb_diag d;
        pfgb_status s = pfgb_diagnostics(ctx, &d);
        if (s != PFGB_OK) return s;
        if (std::isfinite(vf_override)) d.vf_precip = vf_override;   // minimize: mean_h of the iteration
        double R_avg = 0.0;
        if (d.n_if > 0.0) {
            const double ratio = d.n_in / (d.n_if / (P.ic_phi_iface_w * 2.0));
            R_avg = (P.Ny == 2 ? 2.0 : 3.0) * P.dx * ratio;
        }
        const double t = step * P.dt, t_real = t * P.t_real_unit;
        if (csv) {
            fprintf(csv, "%d,%.8f,%.8e,%.8e,%.8e\n", step + csv_step_off, t + csv_t_off, t_real + csv_tr_off,
                    d.vf_precip, R_avg);
            fflush(csv);
        }
        printf("%s step=%05d t=%.6f t_real=%.6e s <x_B_tot>=%.6e vf_precip=%.6e R_avg_internal=%.6e "
               "R_avg_nm=%.6e xB_range=[%.4f, %.4f] t_wall=%s\n",
               dim, step, t, t_real, d.mass_xBtot / (double)N, d.vf_precip, R_avg, R_avg * unit_to_nm, d.xB_min,
               d.xB_max, now_str().c_str());
        return PFGB_OK;
    };

    if ((st = read_state()) != PFGB_OK) { pfgb_destroy(ctx); return fail(st, "pfgb_read_fields"); }
    // initial files (main_cuda.cu:27475-27530): minimize writes phi (and, in
    // the full model, xB) with the case tag; dynamics writes xBtot_0 (and
    // xBtot_gp_init in gp_zone), phi_init, eta_init (gp_zone) and xB_0
    if (minimize) {
        write_vtk(case_dir + "/phi_init_" + tag + ".vtk", "phi", f_phi, P.Nx, P.Ny, P.Nz);
        if (P.minimize_full_model) write_vtk(case_dir + "/xB_init_" + tag + ".vtk", "xB", f_xB, P.Nx, P.Ny, P.Nz);
    } else {
        // recompute_host_xBtot_field (main_cuda.cu:19147-19170)
        for (size_t i = 0; i < N; ++i) {
            const double pc = std::min(std::max(f_phi[i], 0.0), 1.0);
            const double h = h_of(pc);
            const double x = std::min(std::max(f_xB[i], P.xB_eps), 1.0 - P.xB_eps);
            if (gpc) {
                const double he = h_of(std::min(std::max(f_eta[i], 0.0), 1.0));
                f_xBtot[i] = (1.0 - h) * (1.0 - he) * x + (1.0 - h) * he * P.gp_xB_fixed + h;
            } else {
                f_xBtot[i] = (1.0 - h) * x + h;   // the host form adds h_beta alone
            }
        }
        write_vtk(case_dir + xbt_stem + "_0.vtk", xbt_name, f_xBtot, P.Nx, P.Ny, P.Nz);
        if (gp) write_vtk(case_dir + "/xBtot_gp_init.vtk", "xBtot_gp", f_xBtot, P.Nx, P.Ny, P.Nz);
        write_vtk(case_dir + "/phi_init.vtk", "phi", f_phi, P.Nx, P.Ny, P.Nz);
        if (gp) write_vtk(case_dir + "/eta_init.vtk", "eta", f_eta, P.Nx, P.Ny, P.Nz);
        write_vtk(case_dir + "/xB_0.vtk", "xB", f_xB, P.Nx, P.Ny, P.Nz);
    }
    // a continuation writes no step-0 row (main_cuda.cu:28309)
    if (!c.cont && (st = csv_row(0, NAN)) != PFGB_OK) { pfgb_destroy(ctx); return fail(st, "pfgb_diagnostics"); }

    std::vector<double> wall;
    wall.reserve(c.nsteps);
    const auto t0 = std::chrono::steady_clock::now();
    int rc = 0;
    unsigned long long accepted_zm = (unsigned long long)(first_step - 1);
    for (int step = 1; step <= c.nsteps && minimize; ++step) {
        pfgb_min_stats m;
        const auto a = std::chrono::steady_clock::now();
        st = pfgb_minimize(ctx, 1, 1, &m);
        if (st == PFGB_OK) st = pfgb_sync(ctx);
        const double w = std::chrono::duration<double>(std::chrono::steady_clock::now() - a).count();
        if (st != PFGB_OK) { rc = fail(st, "pfgb_minimize"); break; }
        wall.push_back(w);
        fprintf(efp, "%d,%.8e,%.8e,%.8e,%.8e,%.8e,%.8e,%.8e,%.8e,%.8e,%.8e,%.8e,%.8e,%.8e,%.8e,%.8e,%.8e,%.8e,"
                     "%.17e,%.17e,%.17e,%.17e,%d\n",
                step + energy_off, P.dt, m.mean_h, m.V0_target, m.lambda_vol, m.F_surf, m.F_el, m.F_chem_excess,
                m.F_total_excess, m.F_chem_CNT, m.F_total_CNT, m.total_interface_sum, m.total_el_core_sum,
                m.rms_res, m.rms_dphi, m.rms_dY, m.energy_diff_rel, m.vol_err_rel, NAN, NAN, NAN, NAN,
                P.minimize_post_projection_iters);
        fflush(efp);
        if (etrace) {
            fprintf(etrace, "%d,%d,%d,%.17e,%d,%d,%.17e,%.9f,%llu\n", step, step > 1 ? 1 : 0, m.elastic_iterations,
                    m.elastic_relative_residual, m.elastic_relative_residual <= P.elastic_residual_tolerance ? 1 : 0,
                    P.elastic_iter_max, P.elastic_residual_tolerance, w, (unsigned long long)(step - 1));
            fflush(etrace);
        }
        if (step % c.csv_out_every == 0 && (st = csv_row(step, m.mean_h)) != PFGB_OK) {
            rc = fail(st, "pfgb_diagnostics");
            break;
        }
        if (m.converged) {
            printf("[minimize] converged at iter %d (%s)\n", m.converged_iteration, m.condA ? "condA" : "condB");
            break;
        }
    }
    // final audits of the accelerated elastic solver and the zero mode
    // (main_cuda.cu:34300-34350, 34796-34800)
    unsigned long long el_nonconv = 0, el_iters_total = 0, el_last_iters = 0;
    double el_last_resid = NAN, zm_target = NAN;
    for (int step = first_step; step <= c.nsteps && !minimize; ++step) {
        pfgb_step_stats s;
        const auto a = std::chrono::steady_clock::now();
        st = pfgb_step(ctx, 1, &s);
        if (st == PFGB_OK) st = pfgb_sync(ctx);
        const double w = std::chrono::duration<double>(std::chrono::steady_clock::now() - a).count();
        if (st != PFGB_OK) { rc = fail(st, "pfgb_step"); break; }
        wall.push_back(w);
        if (P.pf_y_update_mode == PFGB_Y_Q_TRANSPORT_SPLIT) {
            // the q split's events, as the reference prints them (main_cuda.cu:30262-30266, 30701-30706)
            if (s.q_phase_rejected)
                printf("PF_Q_PHASE_SUBSTEP_REJECTED step=%d policy=rollback_entire_phi_substep\n", step);
            if (s.q_redistributed_cells)
                printf("PF_Q_TRANSPORT_LOCAL_REDISTRIBUTION step=%d violating_cells=%d global_mass_loss=0\n", step,
                       s.q_redistributed_cells);
        }
        if (accel) {
            el_nonconv += s.elastic_converged ? 0 : 1;
            el_iters_total += (unsigned long long)s.elastic_iterations;
            el_last_iters = (unsigned long long)s.elastic_iterations;
            el_last_resid = s.elastic_relative_residual;
        }
        if (P.zero_mode_enabled) zm_target = s.zero_mode_target_mass;
        if (etrace) {
            fprintf(etrace, "%d,%d,%d,%.17e,%d,%d,%.17e,%.9f,%llu\n", step, s.elastic_warm_start_used,
                    s.elastic_iterations, s.elastic_relative_residual, s.elastic_converged, P.elastic_iter_max,
                    P.elastic_residual_tolerance, w, (unsigned long long)(step - 1));
            fflush(etrace);
        }
        if (ztrace) {
            ++accepted_zm;
            fprintf(ztrace, "%d,%.17e,%.17e,%.17e,%.17e,%d,%d,%d,%.17e,%.17e,%.17e,%.17e,%llu\n", step,
                    s.zero_mode_target_mass, s.zero_mode_lambda, s.zero_mode_residual, NAN, s.zero_mode_iterations,
                    s.zero_mode_newton_steps, s.zero_mode_bisection_steps, NAN, NAN, NAN, NAN, accepted_zm);
            fflush(ztrace);
        }
        if (step % c.csv_out_every == 0 && (st = csv_row(step, NAN)) != PFGB_OK) { rc = fail(st, "pfgb_diagnostics"); break; }
        if (step % c.out_every == 0) {
            if ((st = read_state()) != PFGB_OK) { rc = fail(st, "pfgb_read_fields"); break; }
            vtk_set(("_" + std::to_string(step)).c_str(), step);
        }
        if (c.ckpt_every > 0 && (step % c.ckpt_every == 0 || step == c.nsteps)) {   // main_cuda.cu:33494-33560
            st = pfgb_checkpoint_save(ctx, c.ckpt_path.c_str(), c.isc.c_str(), c.fsha.c_str(), c.psha.c_str());
            if (st != PFGB_OK) { rc = fail(st, "PF zero-mode checkpoint write"); break; }
            printf("PF_ZERO_MODE_CHECKPOINT_WRITTEN step=%d path=%s\n", step, c.ckpt_path.c_str());
        }
    }
    const double total = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    int audit_rc = 0;
    if (rc == 0 && !minimize && P.zero_mode_enabled) {
        pfgb_diag zd;
        if ((st = pfgb_diagnostics(ctx, &zd)) != PFGB_OK) rc = fail(st, "pfgb_diagnostics");
        else {
            const double mean_err = (zd.mass_xBtot - zm_target) / (double)N;
            const bool ok = std::isfinite(zd.mass_xBtot) && std::fabs(mean_err) <= 1.0e-10;
            printf("PF_ZERO_MODE_FINAL_AUDIT status=%s final_step=%d target_mass_code=%.17e final_mass_code=%.17e "
                   "mean_mass_error=%.17e gp_paths_enabled=false\n",
                   ok ? "PASS" : "FAIL", c.nsteps, zm_target, zd.mass_xBtot, mean_err);
            if (!ok) audit_rc = 2;
        }
    }
    if (rc == 0 && !minimize && accel) {
        const double n = (double)wall.size();
        printf("PF_ELASTIC_SOLVER_FINAL_AUDIT status=%s mode=ELASTIC_WARM_START_RESIDUAL_V1 steps=%zu "
               "total_iterations=%llu mean_iterations=%.9f last_iterations=%llu last_residual=%.17e "
               "nonconverged_steps=%llu\n",
               el_nonconv == 0 ? "PASS" : "FAIL", wall.size(), el_iters_total, n > 0 ? el_iters_total / n : 0.0,
               el_last_iters, el_last_resid, el_nonconv);
        printf("elastic_solver_status=%s\n", el_nonconv == 0 ? "PASS_ELASTIC_WARM_START_RESIDUAL_V1"
                                                               : "FAIL_ELASTIC_WARM_START_RESIDUAL_V1");
        if (el_nonconv != 0) audit_rc = 2;   // the run completes; the exit status reports it
    }
    if (rc == 0) {
        if ((st = read_state()) != PFGB_OK) rc = fail(st, "pfgb_read_fields");
        else if (minimize) {   // main_cuda.cu:33635-33665
            write_vtk(case_dir + "/phi_final_" + tag + ".vtk", "phi", f_phi, P.Nx, P.Ny, P.Nz, c.nsteps);
            if (P.minimize_full_model)
                write_vtk(case_dir + "/xB_final_" + tag + ".vtk", "xB", f_xB, P.Nx, P.Ny, P.Nz, c.nsteps);
        } else if (c.nsteps % c.out_every != 0) {
            // the last step off the output schedule, numbered nsteps / out_every + 1
            // (main_cuda.cu:33815-33840)
            const int os = c.nsteps / c.out_every + 1;
            vtk_set(("_" + std::to_string(os)).c_str(), os);
        }
    }
    if (csv) fclose(csv);
    if (efp) fclose(efp);
    if (etrace) fclose(etrace);
    if (ztrace) fclose(ztrace);

    // ---- performance summary (write_performance_summary_json, main_cuda.cu:3790) ----
    std::vector<double> sorted = wall;
    std::sort(sorted.begin(), sorted.end());
    const double n = (double)wall.size();
    double avg = 0.0, warm = 0.0;
    for (double x : wall) avg += x;
    avg = n > 0 ? avg / n : NAN;
    for (size_t i = 1; i < wall.size(); ++i) warm += wall[i];
    warm = wall.size() > 1 ? warm / (n - 1) : avg;
    const double med = sorted.empty() ? NAN : sorted[sorted.size() / 2];
    FILE *pj = fopen((case_dir + "/performance_summary.json").c_str(), "w");
    if (pj) {
        fprintf(pj,
                "{\n  \"case_name\": \"%s\",\n  \"picard_enabled\": %.17e,\n  \"picard_iters\": %.17e,\n"
                "  \"picard_omega\": %.17e,\n  \"nsteps\": %.17e,\n  \"dt\": %.17e,\n  \"total_walltime_s\": %.17e,\n"
                "  \"avg_walltime_per_step_s\": %.17e,\n  \"median_walltime_per_step_s\": %.17e,\n"
                "  \"min_walltime_per_step_s\": %.17e,\n  \"max_walltime_per_step_s\": %.17e,\n"
                "  \"warmup_excluded_avg_walltime_per_step_s\": %.17e,\n  \"estimated_steps_per_hour\": %.17e,\n"
                "  \"relative_slowdown_vs_baseline\": %.17e\n}\n",
                tag.c_str(), 0.0, 1.0, 1.0, (double)c.nsteps, P.dt, total, avg, med,
                sorted.empty() ? NAN : sorted.front(), sorted.empty() ? NAN : sorted.back(), warm,
                warm > 0 ? 3600.0 / warm : NAN, NAN);
        fclose(pj);
    }
    FILE *sm = fopen((case_dir + "/summary.txt").c_str(), "w");
    if (sm) {
        fprintf(sm, "case=%s\ngrid=%dx%dx%d\ndt=%.17g\nnsteps=%d\nsteps_done=%zu\nprecision=%s\n", tag.c_str(), P.Nx,
                P.Ny, P.Nz, P.dt, c.nsteps, wall.size(), P.precision == PFGB_PREC_FP32 ? "fp32" : "fp64");
        fprintf(sm, "total_walltime_s=%.6f\nMpts_per_s=%.6f\nexit_status=%d\n", total,
                total > 0 ? (double)N * wall.size() / total / 1e6 : 0.0, rc);
        fclose(sm);
    }
    printf("done: %zu steps, %.3f s, %.3f Mpts/s\n", wall.size(), total,
           total > 0 ? (double)N * wall.size() / total / 1e6 : 0.0);
    pfgb_destroy(ctx);
    return rc != 0 ? rc : audit_rc;
}
