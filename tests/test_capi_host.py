"""C-ABI library: loads without a GPU, exports every declared entry point,
and its host-side logic (defaults, parameter files, derived thermo, raw-field
preparation) matches the reference rules.  No device compute here."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import GOLDEN, REPO


def declared_functions():
    src = open(os.path.join(REPO, "include", "pfgb.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(pfgb_[a-z0-9_]+)\s*\(", src)))


def test_every_declared_symbol_is_exported(capi):
    lib = capi.load()
    names = declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n
    # and the ctypes binding covers the whole header
    assert sorted(n for n, _, _ in capi.EXPORTS) == names


def test_params_struct_size(capi):
    assert capi.load().pfgb_params_size() == ctypes.sizeof(capi.Params)


def test_defaults_follow_reference(capi):
    p = capi.default_params()
    # params_default, main_cuda.cu:15781-16439
    assert p.Y_clip == 20.0 and p.xB_eps == 1e-8 and p.dt == 1e-2
    assert p.elastic_iter_max == 32 and p.elastic_iter_min == 2
    assert p.elastic_residual_tolerance == 1e-6 and p.elastic_warm_start_enabled == 1
    assert p.zero_mode_tolerance_relative == 1e-12 and p.zero_mode_max_iterations == 24
    assert p.thermo_convex_extrapolation_enabled == 0 and p.Y_rhs_term_h_scale == 1.0
    assert p.gp_xB_fixed == pytest.approx(0.3529411764705882)


def test_load_param_file(capi):
    p = capi.load_params_file(os.path.join(GOLDEN, "c2.params"))
    assert p.D_alpha == pytest.approx(625.0) and p.kappa_phi == pytest.approx(3.125)
    assert p.S[0] == pytest.approx(267.85714285714283) and p.S_p[0] == pytest.approx(-119.04761904761904)
    assert p.eps00[0] == pytest.approx(0.046) and p.eps00[1] == pytest.approx(-0.022)
    assert p.gp_W_eta == pytest.approx(1.4880952380952381)
    assert p.pf_params_schema_version == 1


def _write(tmp_path, text):
    f = tmp_path / "x.params"
    f.write_text(text)
    return str(f)


def test_missing_required_key_is_an_error(capi, tmp_path):
    lines = [l for l in open(os.path.join(GOLDEN, "c1.params")) if not l.startswith("S_p_66")]
    with pytest.raises(capi.PfgbError) as e:
        capi.load_params_file(_write(tmp_path, "".join(lines)))
    assert "S_p_" in str(e.value)


def test_bad_number_is_an_error(capi, tmp_path):
    txt = open(os.path.join(GOLDEN, "c1.params")).read().replace("W=1.0", "W=1.0x")
    with pytest.raises(capi.PfgbError) as e:
        capi.load_params_file(_write(tmp_path, txt))
    assert "W" in str(e.value)


def test_unknown_key_warns_and_is_ignored(capi, tmp_path, capfd):
    txt = open(os.path.join(GOLDEN, "c1.params")).read() + "\nnot_a_key = 3 # comment\n"
    p = capi.load_params_file(_write(tmp_path, txt))
    assert p.W == 1.0
    assert "unknown key ignored: not_a_key" in capfd.readouterr().err


@pytest.mark.parametrize("line", ["enable_Y_rhs_picard = 1",
                                  "gp_nuc_enabled = 1", "diagnostic_rsmd_enabled = 1",
                                  "enable_gp_assisted_beta_nucleation = 1"])
def test_unbuilt_path_selectors_are_refused(capi, tmp_path, line):
    base = open(os.path.join(GOLDEN, "c1.params")).read()
    with pytest.raises(capi.PfgbError) as e:
        capi.load_params_file(_write(tmp_path, base + "\n" + line + "\n"))
    assert "not built" in str(e.value)
    # the default value is accepted
    key = line.split("=")[0].strip()
    capi.load_params_file(_write(tmp_path, base + "\n%s = 0\n" % key))


def test_mass_projection_key(capi, tmp_path):
    """y_update_mass_projection_enabled = 1 is accepted (on this path the
    reference's projection never arms) and refused, as in the reference,
    with the zero mode and the conservative composition modes."""
    base = open(os.path.join(GOLDEN, "c2.params")).read()
    p = capi.load_params_file(_write(tmp_path, base + "\ny_update_mass_projection_enabled = 1\n"))
    assert p.y_update_mass_projection_enabled == 1
    for over in (dict(zero_mode_enabled=1), dict(pf_composition_mode=1)):
        q = capi.load_params_file(_write(tmp_path, base + "\ny_update_mass_projection_enabled = 1\n"))
        for k, v in over.items():
            setattr(q, k, v)
        capi.finalize(q)
        ctx = ctypes.c_void_p()
        assert capi.load().pfgb_create(ctypes.byref(q), 0, ctypes.byref(ctx)) == 1
        assert not ctx.value


def test_gp_storage_coupling_keys(capi, tmp_path):
    base = open(os.path.join(GOLDEN, "c2.params")).read()
    p = capi.load_params_file(_write(tmp_path, base + "\ngp_barrier_only_mode = 0\n"))
    assert p.gp_barrier_only_mode == 0 and p.enable_legacy_gp_storage_coupling == 0
    d = capi.default_params()
    assert d.gp_barrier_only_mode == 1
    assert (d.gp_y_update_mode, d.gp_eta_mass_limiter, d.gp_y_picard_iters) == (capi.GP_Y_OLD_RHS,
                                                                                capi.GP_ETA_LIMITER_OFF, 3)
    for text, mode in (("old_rhs", capi.GP_Y_OLD_RHS), ("conservative_y_rhs", capi.GP_Y_CONSERVATIVE_RHS),
                       ("picard_storage", capi.GP_Y_PICARD_STORAGE), ("storage_exact", capi.GP_Y_STORAGE_EXACT)):
        p = capi.load_params_file(_write(tmp_path, base + "\ngp_y_update_mode = %s\n"
                                         "gp_eta_mass_limiter = local_clip\ngp_y_picard_iters = 5\n" % text))
        assert (p.gp_y_update_mode, p.gp_eta_mass_limiter, p.gp_y_picard_iters) == (mode,
                                                                                    capi.GP_ETA_LIMITER_LOCAL_CLIP, 5)
    for line in ("gp_y_update_mode = explicit", "gp_eta_mass_limiter = hard"):
        with pytest.raises(capi.PfgbError):
            capi.load_params_file(_write(tmp_path, base + "\n" + line + "\n"))


def test_y_update_mode_key(capi, tmp_path):
    base = open(os.path.join(GOLDEN, "c1.params")).read()
    p = capi.load_params_file(_write(tmp_path, base + "\npf_y_update_mode = storage_exact\ngp_h_alpha_eps = 1e-6\n"))
    assert p.pf_y_update_mode == capi.Y_STORAGE_EXACT and p.gp_h_alpha_eps == 1e-6
    assert capi.default_params().pf_y_update_mode == capi.Y_LAGGED_RHS
    p = capi.load_params_file(_write(tmp_path, base + "\npf_y_update_mode = x_transport_projection_split\n"
                                     "pf_matrix_storage_floor = 0.2\n"))
    assert p.pf_y_update_mode == capi.Y_X_TRANSPORT_SPLIT and p.pf_matrix_storage_floor == 0.2
    assert p.pf_composition_stabilizer_Dalpha_multiplier == 10.0
    p = capi.load_params_file(_write(tmp_path, base + "\npf_y_update_mode = q_transport_projection_split\n"))
    assert p.pf_y_update_mode == capi.Y_Q_TRANSPORT_SPLIT
    # an unknown mode is refused, not silently replaced
    with pytest.raises(capi.PfgbError) as e:
        capi.load_params_file(_write(tmp_path, base + "\npf_y_update_mode = q_transport\n"))
    assert "pf_y_update_mode" in str(e.value)


def test_composition_mode_keys(capi, tmp_path):
    base = open(os.path.join(GOLDEN, "c1.params")).read()
    p = capi.load_params_file(_write(tmp_path, base + "\npf_composition_mode = qalpha_conservative_local_transaction\n"
                                     "pf_conservative_flux_strategy = pairwise_backward_euler\n"
                                     "pf_conservative_bound_tol = 1e-11\npf_conservative_max_subcycles = 8\n"))
    assert p.pf_composition_mode == capi.COMPOSITION_QALPHA
    assert p.pf_conservative_flux_strategy == capi.CONS_FLUX_BACKWARD_EULER
    assert p.pf_conservative_bound_tol == 1e-11 and p.pf_conservative_max_subcycles == 8
    d = capi.default_params()
    assert d.pf_composition_mode == capi.COMPOSITION_LEGACY
    assert (d.pf_conservative_bound_tol, d.pf_conservative_mass_tol, d.pf_conservative_beta_support_eps,
            d.pf_conservative_max_subcycles) == (1e-12, 1e-10, 1e-10, 64)
    with pytest.raises(capi.PfgbError):
        capi.load_params_file(_write(tmp_path, base + "\npf_composition_mode = ctot\n"))


def test_finalize_matches_oracle(capi, oracle):
    import oracle_py
    p = capi.load_params_file(os.path.join(GOLDEN, "c2.params"))
    capi.finalize(p)
    q = capi.load_params_file(os.path.join(GOLDEN, "c2.params"))
    oracle_py.lib().pfo_params_finalize(ctypes.byref(q))
    assert p.temperature_K == q.temperature_K
    assert p.xB_eq_matrix == q.xB_eq_matrix
    assert p.mu0_compound == pytest.approx(q.mu0_compound, rel=1e-14)


def test_prepare_raw_fields_rules(capi):
    p = capi.default_params()
    phi = np.array([-0.2, 0.5, 1.3])
    xB = np.array([0.0, 0.5, 0.9])
    eta = np.array([2.0, -1.0, 0.25])
    st = capi.load().pfgb_prepare_raw_fields(ctypes.byref(p), 0.34, phi.ctypes.data, xB.ctypes.data,
                                             eta.ctypes.data, None, 3)
    assert st == 0
    assert phi.tolist() == [0.0, 0.5, 1.0] and eta.tolist() == [1.0, 0.0, 0.25]
    assert xB.tolist() == [1e-8, 0.34, 0.34]
    bad = np.array([np.nan, 0, 0])
    st = capi.load().pfgb_prepare_raw_fields(ctypes.byref(p), 0.34, bad.ctypes.data, xB.ctypes.data,
                                             None, None, 3)
    assert st == 6


def test_create_rejects_bad_grid_without_touching_gpu(capi):
    p = capi.default_params()
    p.Nx = 0
    ctx = ctypes.c_void_p()
    assert capi.load().pfgb_create(ctypes.byref(p), 0, ctypes.byref(ctx)) == 1


@pytest.mark.parametrize("over", [dict(model_mode=1, gp_barrier_only_mode=0, mode=1),
                                  dict(model_mode=1, enable_legacy_gp_storage_coupling=1, mode=1),
                                  dict(model_mode=1, gp_barrier_only_mode=0, gp_y_update_mode=4),
                                  dict(model_mode=1, gp_barrier_only_mode=0, gp_eta_mass_limiter=2),
                                  dict(pf_y_update_mode=1, zero_mode_enabled=1),
                                  dict(pf_y_update_mode=2, mode=1),
                                  dict(pf_y_update_mode=2, pf_matrix_storage_floor=0.0),
                                  dict(pf_y_update_mode=3, zero_mode_enabled=1),
                                  dict(pf_y_update_mode=3, mode=1),
                                  dict(pf_y_update_mode=3, model_mode=1),
                                  dict(pf_y_update_mode=4),
                                  dict(pf_composition_mode=1, zero_mode_enabled=1),
                                  dict(pf_composition_mode=2, model_mode=1),
                                  dict(pf_composition_mode=1, mode=1),
                                  dict(pf_composition_mode=1, pf_y_update_mode=1),
                                  dict(pf_composition_mode=2, Nz=15),
                                  dict(pf_composition_mode=1, pf_conservative_bound_tol=0.0),
                                  dict(pf_composition_mode=3)])
def test_create_refuses_unbuilt_or_invalid_composition_paths(capi, over):
    """Refused by the parameter check before any device work."""
    p = capi.load_params_file(os.path.join(GOLDEN, "c2.params"))
    for k, v in over.items():
        setattr(p, k, v)
    capi.finalize(p)
    ctx = ctypes.c_void_p()
    assert capi.load().pfgb_create(ctypes.byref(p), 0, ctypes.byref(ctx)) in (1, 8)
    assert not ctx.value
