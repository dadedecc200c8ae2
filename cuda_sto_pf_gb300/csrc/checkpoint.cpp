// checkpoint.cpp — the reference's zero-mode checkpoint files, so runs can
// hand off to and from its main_cuda (pf_zero_mode_checkpoint.cpp,
// main_cuda.cu:27340-27400 restore, 33494-33560 write).
//
// File = header, then the payload: phi, Y, xB, dY_dt_prev (float64, N each)
// and, in V4, the elastic warm state u_k (complex float, 3 x Nk packed
// ux | uy | uz, the half spectrum [Nx][Ny][Nz/2+1]).  Header fields are
// stored in the order below in native (little-endian) layout, without
// padding:
//   magic[8] "PFZMCHK<v>", u32 version, u32 header_bytes, u64 element_count,
//   [V4: u64 k_element_count], u64 accepted_step, i32 nx, ny, nz,
//   i32 reserved (V4: elastic_state_present), f64 dt_code, temperature_K,
//   target_mass_code, last_lambda, last_residual_code, last_derivative_code,
//   u64 last_iterations, accepted_zero_mode_steps, parameter_fingerprint,
//   [V4: u64 elastic_solver_fingerprint, elastic_source_field_step,
//        elastic_last_iterations, f64 elastic_last_relative_residual],
//   six 64-byte selectors (zero_mode, backend, composition_mode,
//   y_update_mode, explicit_context, reaction_discretization) [V4: and
//   elastic_solver_mode], [V3, V4: three 96-byte identities
//   (initial_state_class, fixture_manifest_sha256,
//   profile_library_manifest_sha256)], u64 payload_checksum.
// Sizes: V2 512, V3 800, V4 904 bytes.  payload_checksum is FNV-1a 64 over
// the header with the checksum field zero, continued over the payload.
// Writes go to "<path>.tmp", renamed into place once the checksum is final.
// This file writes V3 (no elastic state) or V4 and reads V2-V4.
#include <cerrno>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/pfgb.h"

void pfgb_set_error_msg(const char *fmt, ...);

namespace {

constexpr size_t kSel = 64, kIdent = 96;
constexpr size_t kHeaderV2 = 512, kHeaderV3 = 800, kHeaderV4 = 904;
constexpr uint64_t kFnvSeed = 1469598103934665603ULL, kFnvPrime = 1099511628211ULL;

const char *const kZeroModeV1 = "PF_CONSERVED_Y_ZERO_MODE_V1";
const char *const kBackendV1 = "HOST_NEWTON_BISECTION_V1";
const char *const kExplicitContextV1 = "SM_EXPLICIT_CONTEXT_N_V1";
const char *const kReactionTangentV1 = "SM_TANGENT_N_V1";
const char *const kLegacy = "LEGACY_UNSPECIFIED";
const char *const kElasticNotRequired = "ELASTIC_RUNTIME_STATE_NOT_REQUIRED";
const char *const kElasticWarmResidualV1 = "ELASTIC_WARM_START_RESIDUAL_V1";
// the composition path this library builds
const char *const kCompositionLegacy = "legacy";
const char *const kYUpdateLagged = "lagged_rhs";

uint64_t fnv(const void *data, size_t n, uint64_t h) {
    const unsigned char *b = static_cast<const unsigned char *>(data);
    for (size_t i = 0; i < n; ++i) {
        h ^= (uint64_t)b[i];
        h *= kFnvPrime;
    }
    return h;
}

// header bytes, field by field
struct Out {
    std::vector<unsigned char> b;
    template <typename T> void put(T v) {
        unsigned char t[sizeof(T)];
        std::memcpy(t, &v, sizeof(T));
        b.insert(b.end(), t, t + sizeof(T));
    }
    void put_text(const char *s, size_t width) {
        const size_t n = std::strlen(s);
        b.insert(b.end(), s, s + n);
        b.insert(b.end(), width - n, 0);
    }
};
struct In {
    const unsigned char *p;
    size_t off = 0;
    template <typename T> T get() {
        T v;
        std::memcpy(&v, p + off, sizeof(T));
        off += sizeof(T);
        return v;
    }
    const char *text(size_t width) {
        const char *s = reinterpret_cast<const char *>(p + off);
        off += width;
        return s;
    }
};

bool fail(const char *msg) {
    pfgb_set_error_msg("checkpoint: %s", msg);
    return false;
}

// a selector / identity is stored NUL-padded; it must be non-empty and leave room for the NUL
bool text_ok(const char *s, size_t width) {
    const size_t n = strnlen(s, width);
    return n > 0 && n < width;
}
// the stored text equals expected exactly (same rule as the reader of the reference)
bool text_equal(const char *disk, const char *expected, size_t width) {
    const size_t n = strnlen(expected, width);
    return n < width && std::strncmp(disk, expected, width) == 0 && disk[n] == '\0';
}

bool elastic_expected(const pfgb_checkpoint_provenance &p) {
    return std::strcmp(p.elastic_solver_mode, kElasticNotRequired) != 0 || p.elastic_solver_fingerprint != 0;
}

bool all_finite(const double *v, size_t n) {
    for (size_t i = 0; i < n; ++i)
        if (!std::isfinite(v[i])) return false;
    return true;
}
bool all_finite_f(const float *v, size_t n) {
    for (size_t i = 0; i < n; ++i)
        if (!std::isfinite(v[i])) return false;
    return true;
}

size_t cells(const pfgb_checkpoint_state &s) { return (size_t)s.nx * s.ny * s.nz; }
size_t kcells(const pfgb_checkpoint_state &s) { return (size_t)s.nx * s.ny * (s.nz / 2 + 1); }

// the checks of the reference's validate_checkpoint
bool validate(const pfgb_checkpoint_state &s) {
    if (s.nx <= 0 || s.ny <= 0 || s.nz <= 0) return fail("grid dimensions are invalid");
    if (!s.phi || !s.Y || !s.xB || !s.dY_dt_prev) return fail("field buffers missing");
    if (!(s.dt_code > 0.0) || !std::isfinite(s.dt_code) || !(s.temperature_K > 0.0) ||
        !std::isfinite(s.temperature_K))
        return fail("time/temperature is invalid");
    const pfgb_checkpoint_provenance &p = s.provenance;
    if (!text_equal(p.zero_mode, kZeroModeV1, kSel) || !text_ok(p.backend, kSel) ||
        !text_ok(p.composition_mode, kSel) || !text_ok(p.y_update_mode, kSel) || !text_ok(p.explicit_context, kSel) ||
        !text_ok(p.reaction_discretization, kSel) || !text_ok(p.initial_state_class, kIdent) ||
        !text_ok(p.fixture_manifest_sha256, kIdent) || !text_ok(p.profile_library_manifest_sha256, kIdent) ||
        p.parameter_fingerprint == 0)
        return fail("zero-mode provenance is incomplete");
    if (elastic_expected(p) != (s.elastic_present != 0)) return fail("elastic state/provenance presence mismatch");
    if (s.elastic_present) {
        if (!text_equal(p.elastic_solver_mode, kElasticWarmResidualV1, kSel) || p.elastic_solver_fingerprint == 0 ||
            s.accepted_step == 0 || s.elastic_source_field_step + 1 != s.accepted_step || !s.displacement_k ||
            !std::isfinite(s.elastic_last_relative_residual) || s.elastic_last_relative_residual < 0.0 ||
            !all_finite_f(s.displacement_k, 6 * kcells(s)))
            return fail("elastic runtime state is invalid");
    }
    const size_t n = cells(s);
    if (!std::isfinite(s.target_mass_code) || !std::isfinite(s.last_lambda) || !std::isfinite(s.last_residual_code) ||
        !std::isfinite(s.last_derivative_code) || !all_finite(s.phi, n) || !all_finite(s.Y, n) ||
        !all_finite(s.xB, n) || !all_finite(s.dY_dt_prev, n))
        return fail("contains a non-finite value");
    return true;
}

std::vector<unsigned char> header_bytes(const pfgb_checkpoint_state &s, uint64_t checksum) {
    const pfgb_checkpoint_provenance &p = s.provenance;
    const bool v4 = s.elastic_present != 0;
    Out o;
    o.put_text(v4 ? "PFZMCHK4" : "PFZMCHK3", 8);
    o.put<uint32_t>(v4 ? 4u : 3u);
    o.put<uint32_t>((uint32_t)(v4 ? kHeaderV4 : kHeaderV3));
    o.put<uint64_t>(cells(s));
    if (v4) o.put<uint64_t>(kcells(s));
    o.put<uint64_t>(s.accepted_step);
    o.put<int32_t>(s.nx);
    o.put<int32_t>(s.ny);
    o.put<int32_t>(s.nz);
    o.put<int32_t>(v4 ? 1 : 0);
    for (double d : {s.dt_code, s.temperature_K, s.target_mass_code, s.last_lambda, s.last_residual_code,
                     s.last_derivative_code})
        o.put<double>(d);
    o.put<uint64_t>(s.last_iterations);
    o.put<uint64_t>(s.accepted_zero_mode_steps);
    o.put<uint64_t>(p.parameter_fingerprint);
    if (v4) {
        o.put<uint64_t>(p.elastic_solver_fingerprint);
        o.put<uint64_t>(s.elastic_source_field_step);
        o.put<uint64_t>(s.elastic_last_iterations);
        o.put<double>(s.elastic_last_relative_residual);
    }
    for (const char *t : {p.zero_mode, p.backend, p.composition_mode, p.y_update_mode, p.explicit_context,
                          p.reaction_discretization})
        o.put_text(t, kSel);
    if (v4) o.put_text(p.elastic_solver_mode, kSel);
    for (const char *t : {p.initial_state_class, p.fixture_manifest_sha256, p.profile_library_manifest_sha256})
        o.put_text(t, kIdent);
    o.put<uint64_t>(checksum);
    return o.b;
}

bool write_all(FILE *fp, const void *d, size_t n) { return n == 0 || std::fwrite(d, 1, n, fp) == n; }
bool read_all(FILE *fp, void *d, size_t n) { return n == 0 || std::fread(d, 1, n, fp) == n; }

// parsed header of any version
struct Header {
    int version = 0;
    uint64_t element_count = 0, k_element_count = 0, accepted_step = 0;
    int32_t nx = 0, ny = 0, nz = 0, elastic_present = 0;
    double dt_code = 0, temperature_K = 0, target_mass = 0, last_lambda = 0, last_residual = 0, last_derivative = 0;
    uint64_t last_iterations = 0, accepted_zm_steps = 0, parameter_fp = 0, elastic_fp = 0;
    uint64_t elastic_source = 0, elastic_iters = 0;
    double elastic_rel = 0;
    const char *sel[7] = {};
    const char *ident[3] = {};
    uint64_t checksum = 0;
    std::vector<unsigned char> raw;   // header bytes with the checksum field zero
};

bool parse_header(FILE *fp, Header *h) {
    unsigned char prefix[16];
    if (!read_all(fp, prefix, 16)) return fail("header/version mismatch");
    uint32_t version, bytes;
    std::memcpy(&version, prefix + 8, 4);
    std::memcpy(&bytes, prefix + 12, 4);
    const bool m2 = std::memcmp(prefix, "PFZMCHK2", 8) == 0 && version == 2 && bytes == kHeaderV2;
    const bool m3 = std::memcmp(prefix, "PFZMCHK3", 8) == 0 && version == 3 && bytes == kHeaderV3;
    const bool m4 = std::memcmp(prefix, "PFZMCHK4", 8) == 0 && version == 4 && bytes == kHeaderV4;
    if (!m2 && !m3 && !m4) return fail("header/version mismatch");
    h->raw.resize(bytes);
    std::memcpy(h->raw.data(), prefix, 16);
    if (!read_all(fp, h->raw.data() + 16, bytes - 16)) return fail("header/version mismatch");
    h->version = (int)version;
    In in{h->raw.data()};
    in.off = 16;
    h->element_count = in.get<uint64_t>();
    if (m4) h->k_element_count = in.get<uint64_t>();
    h->accepted_step = in.get<uint64_t>();
    h->nx = in.get<int32_t>();
    h->ny = in.get<int32_t>();
    h->nz = in.get<int32_t>();
    h->elastic_present = in.get<int32_t>();
    if (!m4) h->elastic_present = 0;
    h->dt_code = in.get<double>();
    h->temperature_K = in.get<double>();
    h->target_mass = in.get<double>();
    h->last_lambda = in.get<double>();
    h->last_residual = in.get<double>();
    h->last_derivative = in.get<double>();
    h->last_iterations = in.get<uint64_t>();
    h->accepted_zm_steps = in.get<uint64_t>();
    h->parameter_fp = in.get<uint64_t>();
    if (m4) {
        h->elastic_fp = in.get<uint64_t>();
        h->elastic_source = in.get<uint64_t>();
        h->elastic_iters = in.get<uint64_t>();
        h->elastic_rel = in.get<double>();
    }
    const int nsel = m4 ? 7 : 6;
    for (int i = 0; i < nsel; ++i) h->sel[i] = in.text(kSel);
    if (!m2)
        for (int i = 0; i < 3; ++i) h->ident[i] = in.text(kIdent);
    const size_t csum_off = in.off;
    h->checksum = in.get<uint64_t>();
    std::memset(h->raw.data() + csum_off, 0, 8);
    return true;
}

// the reference's read_checkpoint provenance rules per version
bool provenance_matches(const Header &h, const pfgb_checkpoint_provenance &e) {
    const char *exp_sel[6] = {e.zero_mode, e.backend, e.composition_mode, e.y_update_mode, e.explicit_context,
                              e.reaction_discretization};
    const char *exp_id[3] = {e.initial_state_class, e.fixture_manifest_sha256, e.profile_library_manifest_sha256};
    bool ok = h.parameter_fp == e.parameter_fingerprint;
    for (int i = 0; i < 6; ++i) ok = ok && text_equal(h.sel[i], exp_sel[i], kSel);
    if (h.version >= 3)
        for (int i = 0; i < 3; ++i) ok = ok && text_equal(h.ident[i], exp_id[i], kIdent);
    if (h.version == 4)
        ok = ok && h.elastic_present == 1 && elastic_expected(e) &&
             text_equal(h.sel[6], e.elastic_solver_mode, kSel) && h.elastic_fp == e.elastic_solver_fingerprint;
    return ok;
}

bool copy_text(char *dst, size_t width, const char *src) {
    if (!src) src = kLegacy;
    const size_t n = std::strlen(src);
    if (n == 0 || n >= width) return false;
    std::memset(dst, 0, width);
    std::memcpy(dst, src, n);
    return true;
}

}  // namespace

extern "C" {

uint64_t pfgb_fnv1a64(const void *data, size_t size, uint64_t seed) { return fnv(data, size, seed); }

// pf_zero_mode_parameter_fingerprint (main_cuda.cu:4187-4220): FNV-1a over
// the grid, time step, temperature, spacing, molar volumes, mobilities,
// gradient and well coefficients, Y clip, xB guard, the two Y-RHS switches,
// the composition and Y-update mode names and the zero-mode explicit-context
// and reaction-tangent names (each with its NUL).
uint64_t pfgb_parameter_fingerprint(const pfgb_params *p) {
    if (!p) return 0;
    uint64_t h = kFnvSeed;
    auto add = [&](const void *d, size_t n) { h = fnv(d, n, h); };
    const int32_t grid[3] = {p->Nx, p->Ny, p->Nz};
    add(grid, sizeof(grid));
    for (double d : {p->dt, p->temperature_C, p->dx, p->dy, p->dz, p->v_A, p->v_B, p->D_alpha, p->D_compound,
                     p->L_phi, p->kappa_phi, p->W, p->Y_clip, p->xB_eps})
        add(&d, sizeof(d));
    const int32_t flags[2] = {p->enable_Y_rhs_previous_time_level, p->disable_Y_rhs_gamma_term};
    add(flags, sizeof(flags));
    const char *ymode = p->pf_y_update_mode == PFGB_Y_STORAGE_EXACT      ? "storage_exact"
                        : p->pf_y_update_mode == PFGB_Y_X_TRANSPORT_SPLIT ? "x_transport_projection_split"
                        : p->pf_y_update_mode == PFGB_Y_Q_TRANSPORT_SPLIT ? "q_transport_projection_split"
                                                                           : kYUpdateLagged;
    for (const char *s : {kCompositionLegacy, ymode, kExplicitContextV1, kReactionTangentV1})
        add(s, std::strlen(s) + 1);
    return h == 0 ? 1 : h;
}

// elastic_solver_parameter_fingerprint (main_cuda.cu:4223-4264): grid,
// spacing, the five solver switches / limits, tolerance and floor, the
// fail flag, the 21 + 21 stiffness entries and the 13 strain constants.
uint64_t pfgb_elastic_solver_fingerprint(const pfgb_params *p) {
    if (!p) return 0;
    uint64_t h = kFnvSeed;
    auto add = [&](const void *d, size_t n) { h = fnv(d, n, h); };
    const int32_t grid[3] = {p->Nx, p->Ny, p->Nz};
    add(grid, sizeof(grid));
    for (double d : {p->dx, p->dy, p->dz}) add(&d, sizeof(d));
    const int32_t sw[5] = {p->elastic_enabled, p->elastic_warm_start_enabled, p->elastic_residual_control_enabled,
                           p->elastic_iter_min, p->elastic_iter_max};
    add(sw, sizeof(sw));
    for (double d : {p->elastic_residual_tolerance, p->elastic_residual_absolute_floor}) add(&d, sizeof(d));
    const int32_t fail_flag = p->elastic_fail_on_nonconvergence;
    add(&fail_flag, sizeof(fail_flag));
    double stiff[42];
    for (int i = 0; i < 21; ++i) { stiff[i] = p->S[i]; stiff[21 + i] = p->S_p[i]; }
    add(stiff, sizeof(stiff));
    double strain[13];
    for (int i = 0; i < 6; ++i) strain[i] = p->eps00[i];
    strain[6] = p->eps_iso_over_vB;
    for (int i = 0; i < 6; ++i) strain[7 + i] = p->E0[i];
    add(strain, sizeof(strain));
    return h == 0 ? 1 : h;
}

pfgb_status pfgb_checkpoint_provenance_for(const pfgb_params *p, const char *initial_state_class,
                                           const char *fixture_manifest_sha256,
                                           const char *profile_library_manifest_sha256,
                                           pfgb_checkpoint_provenance *out) {
    if (!p || !out) return PFGB_ERR_INVALID;
    std::memset(out, 0, sizeof(*out));
    const bool accel = p->elastic_enabled && (p->elastic_warm_start_enabled || p->elastic_residual_control_enabled);
    bool ok = copy_text(out->zero_mode, kSel, kZeroModeV1) && copy_text(out->backend, kSel, kBackendV1) &&
              copy_text(out->composition_mode, kSel, kCompositionLegacy) &&
              copy_text(out->y_update_mode, kSel, kYUpdateLagged) &&
              copy_text(out->explicit_context, kSel, kExplicitContextV1) &&
              copy_text(out->reaction_discretization, kSel, kReactionTangentV1) &&
              copy_text(out->elastic_solver_mode, kSel, accel ? kElasticWarmResidualV1 : kElasticNotRequired) &&
              copy_text(out->initial_state_class, kIdent, initial_state_class) &&
              copy_text(out->fixture_manifest_sha256, kIdent, fixture_manifest_sha256) &&
              copy_text(out->profile_library_manifest_sha256, kIdent, profile_library_manifest_sha256);
    if (!ok) {
        pfgb_set_error_msg("checkpoint: an identity string is empty or longer than %zu bytes", kIdent - 1);
        return PFGB_ERR_INVALID;
    }
    out->elastic_solver_fingerprint = accel ? pfgb_elastic_solver_fingerprint(p) : 0;
    out->parameter_fingerprint = pfgb_parameter_fingerprint(p);
    return PFGB_OK;
}

pfgb_status pfgb_checkpoint_write_file(const char *path, const pfgb_checkpoint_state *s) {
    if (!path || !s) return PFGB_ERR_INVALID;
    if (!validate(*s)) return PFGB_ERR_INVALID;
    std::vector<unsigned char> head = header_bytes(*s, 0);
    uint64_t csum = fnv(head.data(), head.size(), kFnvSeed);
    const size_t n = cells(*s);
    const double *fields[4] = {s->phi, s->Y, s->xB, s->dY_dt_prev};
    for (const double *f : fields) csum = fnv(f, n * sizeof(double), csum);
    if (s->elastic_present) csum = fnv(s->displacement_k, 6 * kcells(*s) * sizeof(float), csum);
    head = header_bytes(*s, csum);
    const std::string tmp = std::string(path) + ".tmp";
    FILE *fp = std::fopen(tmp.c_str(), "wb");
    if (!fp) {
        pfgb_set_error_msg("checkpoint: cannot open %s: %s", tmp.c_str(), std::strerror(errno));
        return PFGB_ERR_IO;
    }
    bool ok = write_all(fp, head.data(), head.size());
    for (const double *f : fields) ok = ok && write_all(fp, f, n * sizeof(double));
    if (s->elastic_present) ok = ok && write_all(fp, s->displacement_k, 6 * kcells(*s) * sizeof(float));
    ok = (std::fflush(fp) == 0) && ok;
    ok = (std::fclose(fp) == 0) && ok;
    if (!ok) {
        std::remove(tmp.c_str());
        pfgb_set_error_msg("checkpoint: writing %s failed", tmp.c_str());
        return PFGB_ERR_IO;
    }
    if (std::rename(tmp.c_str(), path) != 0) {
        const std::string why = std::strerror(errno);
        std::remove(tmp.c_str());
        pfgb_set_error_msg("checkpoint: atomic rename to %s failed: %s", path, why.c_str());
        return PFGB_ERR_IO;
    }
    return PFGB_OK;
}

pfgb_status pfgb_checkpoint_peek(const char *path, int32_t *version, int32_t *nx, int32_t *ny, int32_t *nz,
                                 int32_t *elastic_present) {
    if (!path) return PFGB_ERR_INVALID;
    FILE *fp = std::fopen(path, "rb");
    if (!fp) {
        pfgb_set_error_msg("checkpoint: cannot open %s: %s", path, std::strerror(errno));
        return PFGB_ERR_IO;
    }
    Header h;
    const bool ok = parse_header(fp, &h);
    std::fclose(fp);
    if (!ok) return PFGB_ERR_IO;
    if (version) *version = h.version;
    if (nx) *nx = h.nx;
    if (ny) *ny = h.ny;
    if (nz) *nz = h.nz;
    if (elastic_present) *elastic_present = h.elastic_present;
    return PFGB_OK;
}

pfgb_status pfgb_checkpoint_read_file(const char *path, const pfgb_checkpoint_provenance *expected,
                                      pfgb_checkpoint_state *s) {
    if (!path || !expected || !s || !s->phi || !s->Y || !s->xB || !s->dY_dt_prev) return PFGB_ERR_INVALID;
    FILE *fp = std::fopen(path, "rb");
    if (!fp) {
        pfgb_set_error_msg("checkpoint: cannot open %s: %s", path, std::strerror(errno));
        return PFGB_ERR_IO;
    }
    Header h;
    auto bad = [&](const char *why, pfgb_status st) {
        std::fclose(fp);
        pfgb_set_error_msg("checkpoint %s rejected: %s", path, why);
        return st;
    };
    if (!parse_header(fp, &h)) return bad("header/version mismatch", PFGB_ERR_IO);
    if (h.version == 3 && elastic_expected(*expected))
        return bad("V3 file lacks the required elastic runtime state", PFGB_ERR_INVALID);
    if (h.version == 2 && (elastic_expected(*expected) || !text_equal(expected->initial_state_class, kLegacy, kIdent) ||
                           !text_equal(expected->fixture_manifest_sha256, kLegacy, kIdent) ||
                           !text_equal(expected->profile_library_manifest_sha256, kLegacy, kIdent)))
        return bad("legacy V2 file lacks the required fixture/library/elastic provenance", PFGB_ERR_INVALID);
    if (!provenance_matches(h, *expected)) return bad("provenance mismatch", PFGB_ERR_INVALID);
    if (h.element_count == 0 || h.nx <= 0 || h.ny <= 0 || h.nz <= 0 ||
        h.element_count != (uint64_t)h.nx * h.ny * h.nz)
        return bad("element count is invalid", PFGB_ERR_IO);
    if (h.nx != s->nx || h.ny != s->ny || h.nz != s->nz) return bad("grid differs from the caller's", PFGB_ERR_INVALID);
    const uint64_t nk = (uint64_t)h.nx * h.ny * (h.nz / 2 + 1);
    if (h.version == 4 && (h.k_element_count != nk || !s->displacement_k))
        return bad("elastic k-space element count is invalid (or no buffer for it)", PFGB_ERR_INVALID);
    uint64_t csum = fnv(h.raw.data(), h.raw.size(), kFnvSeed);
    const size_t n = (size_t)h.element_count;
    double *fields[4] = {s->phi, s->Y, s->xB, s->dY_dt_prev};
    bool ok = true;
    for (double *f : fields) {
        ok = ok && read_all(fp, f, n * sizeof(double));
        if (ok) csum = fnv(f, n * sizeof(double), csum);
    }
    if (h.version == 4) {
        ok = ok && read_all(fp, s->displacement_k, 6 * (size_t)nk * sizeof(float));
        if (ok) csum = fnv(s->displacement_k, 6 * (size_t)nk * sizeof(float), csum);
    }
    unsigned char extra;
    if (ok && std::fread(&extra, 1, 1, fp) != 0) ok = false;
    std::fclose(fp);
    if (!ok || csum != h.checksum) {
        pfgb_set_error_msg("checkpoint %s rejected: payload checksum mismatch", path);
        return PFGB_ERR_IO;
    }
    s->accepted_step = h.accepted_step;
    s->elastic_present = h.version == 4 ? 1 : 0;
    s->dt_code = h.dt_code;
    s->temperature_K = h.temperature_K;
    s->target_mass_code = h.target_mass;
    s->last_lambda = h.last_lambda;
    s->last_residual_code = h.last_residual;
    s->last_derivative_code = h.last_derivative;
    s->last_iterations = h.last_iterations;
    s->accepted_zero_mode_steps = h.accepted_zm_steps;
    s->elastic_source_field_step = h.elastic_source;
    s->elastic_last_iterations = h.elastic_iters;
    s->elastic_last_relative_residual = h.elastic_rel;
    s->provenance = *expected;
    if (!validate(*s)) return PFGB_ERR_INVALID;
    return PFGB_OK;
}

}  // extern "C"
