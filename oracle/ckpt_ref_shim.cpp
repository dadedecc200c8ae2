// ckpt_ref_shim.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Exposes the reference's own zero-mode checkpoint writer and reader
// (pf_zero_mode_checkpoint.cpp, compiled in place from the reference tree
// by `python oracle/build_oracle.py --ref` into oracle/_ref/libpfckpt.so)
// through C entry points that take the flat structs of include/pfgb.h, so
// tests can compare the library's files with the reference's byte for byte
// and read each one's files with the other.  Nothing here is product code.
#include <cstring>
#include <string>

#include "pf_zero_mode_checkpoint.h"
#include "../include/pfgb.h"

namespace {

pf_zero_mode::Provenance to_ref(const pfgb_checkpoint_provenance &p) {
    pf_zero_mode::Provenance r;
    r.zero_mode = p.zero_mode;
    r.backend = p.backend;
    r.composition_mode = p.composition_mode;
    r.y_update_mode = p.y_update_mode;
    r.explicit_context = p.explicit_context;
    r.reaction_discretization = p.reaction_discretization;
    r.initial_state_class = p.initial_state_class;
    r.fixture_manifest_sha256 = p.fixture_manifest_sha256;
    r.profile_library_manifest_sha256 = p.profile_library_manifest_sha256;
    r.elastic_solver_mode = p.elastic_solver_mode;
    r.elastic_solver_fingerprint = p.elastic_solver_fingerprint;
    r.parameter_fingerprint = p.parameter_fingerprint;
    return r;
}

void set_err(char *err, int n, const std::string &m) {
    if (err && n > 0) {
        std::strncpy(err, m.c_str(), (size_t)n - 1);
        err[n - 1] = '\0';
    }
}

}  // namespace

extern "C" int ref_ckpt_write(const char *path, const pfgb_checkpoint_state *s, char *err, int n) {
    pf_zero_mode::Checkpoint c;
    c.accepted_step = s->accepted_step;
    c.nx = s->nx; c.ny = s->ny; c.nz = s->nz;
    c.dt_code = s->dt_code;
    c.temperature_K = s->temperature_K;
    c.provenance = to_ref(s->provenance);
    c.zero_mode.target_mass_code = s->target_mass_code;
    c.zero_mode.last_lambda = s->last_lambda;
    c.zero_mode.last_residual_code = s->last_residual_code;
    c.zero_mode.last_derivative_code = s->last_derivative_code;
    c.zero_mode.last_iterations = s->last_iterations;
    c.zero_mode.accepted_zero_mode_steps = s->accepted_zero_mode_steps;
    const size_t N = (size_t)s->nx * s->ny * s->nz, Nk = (size_t)s->nx * s->ny * (s->nz / 2 + 1);
    c.phi.assign(s->phi, s->phi + N);
    c.Y.assign(s->Y, s->Y + N);
    c.xB.assign(s->xB, s->xB + N);
    c.dY_dt_prev.assign(s->dY_dt_prev, s->dY_dt_prev + N);
    if (s->elastic_present) {
        c.elastic.present = true;
        c.elastic.source_field_step = s->elastic_source_field_step;
        c.elastic.last_iterations = s->elastic_last_iterations;
        c.elastic.last_relative_residual = s->elastic_last_relative_residual;
        c.elastic.displacement_k.assign(s->displacement_k, s->displacement_k + 6 * Nk);
    }
    std::string e;
    const bool ok = pf_zero_mode::write_checkpoint(path, c, &e);
    if (!ok) set_err(err, n, e);
    return ok ? 1 : 0;
}

extern "C" int ref_ckpt_read(const char *path, const pfgb_checkpoint_provenance *expected, pfgb_checkpoint_state *s,
                             char *err, int n) {
    pf_zero_mode::Checkpoint c;
    std::string e;
    if (!pf_zero_mode::read_checkpoint(path, to_ref(*expected), &c, &e)) {
        set_err(err, n, e);
        return 0;
    }
    if (c.nx != s->nx || c.ny != s->ny || c.nz != s->nz) {
        set_err(err, n, "grid differs from the caller's");
        return 0;
    }
    s->accepted_step = c.accepted_step;
    s->dt_code = c.dt_code;
    s->temperature_K = c.temperature_K;
    s->target_mass_code = c.zero_mode.target_mass_code;
    s->last_lambda = c.zero_mode.last_lambda;
    s->last_residual_code = c.zero_mode.last_residual_code;
    s->last_derivative_code = c.zero_mode.last_derivative_code;
    s->last_iterations = c.zero_mode.last_iterations;
    s->accepted_zero_mode_steps = c.zero_mode.accepted_zero_mode_steps;
    s->elastic_present = c.elastic.present ? 1 : 0;
    s->elastic_source_field_step = c.elastic.source_field_step;
    s->elastic_last_iterations = c.elastic.last_iterations;
    s->elastic_last_relative_residual = c.elastic.last_relative_residual;
    std::memcpy(s->phi, c.phi.data(), c.phi.size() * sizeof(double));
    std::memcpy(s->Y, c.Y.data(), c.Y.size() * sizeof(double));
    std::memcpy(s->xB, c.xB.data(), c.xB.size() * sizeof(double));
    std::memcpy(s->dY_dt_prev, c.dY_dt_prev.data(), c.dY_dt_prev.size() * sizeof(double));
    if (c.elastic.present && s->displacement_k)
        std::memcpy(s->displacement_k, c.elastic.displacement_k.data(), c.elastic.displacement_k.size() * sizeof(float));
    return 1;
}
