"""The oracle's per-cell physics against the reference's own kernels.

oracle/_ref/librefk.so is the kernel section of the reference's
cuda_kernels.cu (lines after its includes up to the launch wrappers) built
for the host by oracle/build_oracle.py, with a shim that defines the CUDA
qualifiers away; a launch is a loop over cells, so each value is the
reference kernel's own arithmetic.  The oracle's step functions run on the
same seeded fields through its test hooks.  Skipped where the reference tree
is absent (the library is built only beside it)."""
import ctypes
import os
import sys

import numpy as np
import pytest

from conftest import REPO, params_for

sys.path.insert(0, os.path.join(REPO, "oracle"))

dp = ctypes.POINTER(ctypes.c_double)
fp = ctypes.POINTER(ctypes.c_float)
ip = ctypes.POINTER(ctypes.c_int)


def _refk():
    path = os.path.join(REPO, "oracle", "_ref", "librefk.so")
    if not os.path.exists(path):
        import build_oracle
        path = build_oracle.build_ref_kernels()
    if not path or not os.path.exists(path):
        pytest.skip("reference kernels not built (reference tree absent)")
    L = ctypes.CDLL(path)
    L.refk_set_convex.argtypes = [ctypes.c_int]
    L.refk_phi_rhs.argtypes = [dp, dp, dp, dp, ctypes.c_int, dp, ip, fp, fp, dp, dp]
    L.refk_eta_rhs.argtypes = [dp, dp, dp, dp, ctypes.c_int, dp, ip, fp]
    return L


def _ptr(a, t=dp):
    return a.ctypes.data_as(t)


def _fields(n, seed):
    rng = np.random.default_rng(seed)
    phi = rng.uniform(-0.05, 1.05, n)
    eta = rng.uniform(-0.05, 1.05, n)
    xB = rng.uniform(1e-4, 0.45, n)
    sig = rng.normal(0.0, 0.05, 6 * n).astype(np.float32)
    eps = rng.normal(0.0, 0.01, 6 * n).astype(np.float32)
    return phi, eta, xB, sig, eps


def _oracle_state(capi, p):
    import oracle_py
    o = oracle_py.Oracle(p, threads=1)
    L = o.L
    L.pfo_test_phi_rhs.argtypes = [ctypes.c_void_p, ctypes.c_int, dp, dp, dp, dp, dp, dp]
    L.pfo_test_eta_rhs.argtypes = [ctypes.c_void_p, dp, dp, dp, dp, dp]
    return o


CASES = [
    # (label, model_mode, gp_elastic_enabled, gp_elastic_active_phi, convex)
    ("two_phase", 0, 0, 0, 0),
    ("two_phase_convex", 0, 0, 0, 1),
    ("gp_zone", 1, 0, 0, 0),
    ("gp_zone_gp_elastic", 1, 1, 1, 0),
]


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_phi_rhs_matches_reference_kernel(capi, case):
    _, mm, gel, act, cv = case
    L = _refk()
    n = 8
    p = params_for(capi, "c2.params", n=n, model_mode=mm, gp_elastic_enabled=gel, gp_elastic_active_phi=act,
                   thermo_convex_extrapolation_enabled=cv, elastic_shift_dimless=0.0125)
    N = n ** 3
    phi, eta, xB, sig, eps = _fields(N, 11 + mm + 2 * gel + 4 * cv)
    L.refk_set_convex(cv)
    d = np.array([p.temperature_K, p.mu_reference_scale, p.v_A, p.v_B, p.mu0_compound, p.Vm_compound,
                  p.Vm_alpha_0, p.dVm_alpha_dxB, p.W, p.eps_iso_over_vB, p.gp_eps_iso,
                  p.gp_elastic_derivative_scale, p.elastic_shift_dimless])
    flags = np.array([mm, gel, act, 0, 1], dtype=np.int32)
    Sp = np.array(p.S_p[:])
    e00 = np.array(p.eps00[:])
    ref = np.zeros(N)
    L.refk_phi_rhs(_ptr(phi), _ptr(eta), _ptr(xB), _ptr(ref), N, _ptr(d), _ptr(flags, ip), _ptr(sig, fp),
                   _ptr(eps, fp), _ptr(Sp), _ptr(e00))
    o = _oracle_state(capi, p)
    coupling = 1 if (not (mm and gel) or act) else 0
    got = np.zeros(N)
    o.L.pfo_test_phi_rhs(o.s, coupling, _ptr(phi), _ptr(eta), _ptr(xB), _ptr(sig.astype(np.float64)),
                         _ptr(eps.astype(np.float64)), _ptr(got))
    scale = np.abs(ref).max()
    assert np.abs(got - ref).max() <= 1e-12 * scale, np.abs(got - ref).max() / scale


@pytest.mark.parametrize("gel", [0, 1])
def test_eta_rhs_matches_reference_kernel(capi, gel):
    L = _refk()
    n = 8
    p = params_for(capi, "c2.params", n=n, model_mode=1, gp_elastic_enabled=gel, gp_elastic_active_eta=gel)
    N = n ** 3
    phi, eta, xB, sig, _ = _fields(N, 31 + gel)
    L.refk_set_convex(p.thermo_convex_extrapolation_enabled)
    d = np.array([p.temperature_K, p.mu_reference_scale, p.Vm_alpha_0, p.dVm_alpha_dxB, p.gp_xB_fixed,
                  p.gp_delta_g0, p.gp_W_eta, p.eps_iso_over_vB, p.gp_eps_iso, p.gp_elastic_derivative_scale])
    flags = np.array([gel, gel], dtype=np.int32)
    ref = np.zeros(N)
    L.refk_eta_rhs(_ptr(eta), _ptr(phi), _ptr(xB), _ptr(ref), N, _ptr(d), _ptr(flags, ip), _ptr(sig, fp))
    o = _oracle_state(capi, p)
    got = np.zeros(N)
    o.L.pfo_test_eta_rhs(o.s, _ptr(eta), _ptr(phi), _ptr(xB), _ptr(sig.astype(np.float64)), _ptr(got))
    scale = np.abs(ref).max()
    assert np.abs(got - ref).max() <= 1e-12 * scale, np.abs(got - ref).max() / scale


@pytest.mark.parametrize("gp", [0, 1])
def test_mu_matches_reference_kernel(capi, gp):
    L = _refk()
    L.refk_mu.argtypes = [ctypes.c_int, dp, dp, dp, dp, ctypes.c_int, dp, fp, ctypes.c_int]
    n = 8
    p = params_for(capi, "c2.params", n=n, model_mode=gp)
    N = n ** 3
    rng = np.random.default_rng(41 + gp)
    Y = rng.uniform(-19.0, 3.0, N)
    phi = rng.uniform(-0.05, 1.05, N)
    sig = rng.normal(0.0, 0.05, 6 * N).astype(np.float32)
    L.refk_set_convex(p.thermo_convex_extrapolation_enabled)
    d = np.array([p.temperature_K, p.mu_reference_scale, p.v_A, p.v_B, p.mu0_compound, p.Vm_compound,
                  p.Vm_alpha_0, p.dVm_alpha_dxB, p.Y_clip, p.xB_eps, p.eps_iso_over_vB])
    rx, rmu = np.zeros(N), np.zeros(N)
    L.refk_mu(gp, _ptr(Y), _ptr(phi), _ptr(rx), _ptr(rmu), N, _ptr(d), _ptr(sig, fp), 1)
    o = _oracle_state(capi, p)
    o.L.pfo_test_mu.argtypes = [ctypes.c_void_p, dp, dp, dp, dp, dp]
    gx, gmu = np.zeros(N), np.zeros(N)
    o.L.pfo_test_mu(o.s, _ptr(Y), _ptr(phi), _ptr(sig.astype(np.float64)), _ptr(gx), _ptr(gmu))
    assert np.array_equal(gx, rx) or np.abs(gx - rx).max() <= 1e-15
    assert np.abs(gmu - rmu).max() <= 1e-12 * np.abs(rmu).max()


@pytest.mark.parametrize("form", ["lagged", "previous_level", "no_gamma", "zero_mode"])
def test_y_rhs_matches_reference_kernel(capi, form):
    L = _refk()
    L.refk_y_rhs.argtypes = [ctypes.c_int, dp, dp, dp, dp, dp, dp, dp, ctypes.c_int, dp, ip]
    n = 8
    zm = 1 if form == "zero_mode" else 0
    prev = 1 if form == "previous_level" else 0
    nogam = 1 if form == "no_gamma" else 0
    p = params_for(capi, "c2.params", n=n, zero_mode_enabled=zm, enable_Y_rhs_previous_time_level=prev,
                   disable_Y_rhs_gamma_term=nogam, Y_rhs_term_h_scale=1.0 if form != "lagged" else 0.75)
    N = n ** 3
    rng = np.random.default_rng(53)
    divJ = rng.normal(0.0, 1.0, N)
    phi_new = rng.uniform(0.0, 1.0, N)
    phi_old = np.clip(phi_new + rng.normal(0.0, 0.01, N), 0.0, 1.0)
    lapY = rng.normal(0.0, 0.5, N)
    Y = rng.uniform(-10.0, 2.0, N)
    dYdt = rng.normal(0.0, 0.3, N)
    dt, mean_DY = p.dt, 123.25
    L.refk_set_convex(p.thermo_convex_extrapolation_enabled)
    d = np.array([dt, p.v_B, mean_DY, p.Y_rhs_term_h_scale])
    flags = np.array([prev, nogam], dtype=np.int32)
    ref = np.zeros(N)
    L.refk_y_rhs(zm, _ptr(divJ), _ptr(phi_new), _ptr(phi_old), _ptr(lapY), _ptr(Y), _ptr(dYdt), _ptr(ref), N,
                 _ptr(d), _ptr(flags, ip))
    o = _oracle_state(capi, p)
    o.L.pfo_test_y_rhs.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, dp, dp, dp, dp, dp, dp, dp]
    got = np.zeros(N)
    o.L.pfo_test_y_rhs(o.s, dt, mean_DY, _ptr(divJ), _ptr(phi_new), _ptr(phi_old), _ptr(lapY), _ptr(Y), _ptr(dYdt),
                       _ptr(got))
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()


@pytest.mark.parametrize("mode", ["two_phase", "gp_zone", "gp_zone_gp_elastic"])
def test_polarization_matches_reference_kernel(capi, mode):
    """The elastic iteration's polarization h = C0:eps - C:(eps + E0 - eps0).
    The reference computes it in float arithmetic, the oracle in double with
    float storage, so the bound is float round-off: 1e-5 of the largest
    component."""
    L = _refk()
    L.refk_polarization.argtypes = [fp, dp, dp, dp, fp, ctypes.c_int, fp, fp, fp, fp, dp, ip]
    n = 8
    mm = 0 if mode == "two_phase" else 1
    gel = 1 if mode == "gp_zone_gp_elastic" else 0
    p = params_for(capi, "c2.params", n=n, model_mode=mm, gp_elastic_enabled=gel, elastic_precision=capi.PREC_FP32)
    N = n ** 3
    phi, eta, xB, _, eps = _fields(N, 61 + mm + gel)
    f32 = lambda a: np.array(a[:], dtype=np.float32)   # noqa: E731
    S, Sp, e00, E0 = f32(p.S), f32(p.S_p), f32(p.eps00), f32(p.E0)
    d = np.array([p.eps_iso_over_vB, p.gp_eps_iso])
    flags = np.array([mm, gel], dtype=np.int32)
    ref = np.zeros(6 * N, dtype=np.float32)
    L.refk_polarization(_ptr(eps, fp), _ptr(phi), _ptr(eta), _ptr(xB), _ptr(ref, fp), N, _ptr(S, fp), _ptr(Sp, fp),
                        _ptr(e00, fp), _ptr(E0, fp), _ptr(d), _ptr(flags, ip))
    o = _oracle_state(capi, p)
    o.L.pfo_test_polarization.argtypes = [ctypes.c_void_p, ctypes.c_int, dp, dp, dp, dp, dp]
    got = np.zeros(6 * N)
    o.L.pfo_test_polarization(o.s, 0, _ptr(phi), _ptr(eta), _ptr(xB), _ptr(eps.astype(np.float64)), _ptr(got))
    ref = ref.astype(np.float64)
    assert np.abs(got - ref).max() <= 1e-5 * np.abs(ref).max(), np.abs(got - ref).max() / np.abs(ref).max()


def test_green_matches_reference_kernel(capi):
    """u = -i G(k) (k . tau) of the homogeneous medium, on a non-cubic grid
    (Nyquist planes included); float arithmetic on the reference side."""
    L = _refk()
    L.refk_green.argtypes = [fp, fp, ctypes.c_int, ctypes.c_int, ctypes.c_int, fp, ctypes.c_double,
                             ctypes.c_double, ctypes.c_double]
    Nx, Ny, Nz = 6, 8, 10
    p = params_for(capi, "c2.params", n=8, elastic_precision=capi.PREC_FP32)
    p.Nx, p.Ny, p.Nz = Nx, Ny, Nz
    capi.finalize(p)
    Nk = Nx * Ny * (Nz // 2 + 1)
    rng = np.random.default_rng(71)
    tau = rng.normal(0.0, 1.0, 12 * Nk).astype(np.float32)
    S = np.array(p.S[:], dtype=np.float32)
    ref = np.zeros(6 * Nk, dtype=np.float32)
    L.refk_green(_ptr(tau, fp), _ptr(ref, fp), Nx, Ny, Nz, _ptr(S, fp), p.dx, p.dy, p.dz)
    o = _oracle_state(capi, p)
    o.L.pfo_test_green.argtypes = [ctypes.c_void_p, dp, dp]
    got = np.zeros(6 * Nk)
    o.L.pfo_test_green(o.s, _ptr(tau.astype(np.float64)), _ptr(got))
    ref = ref.astype(np.float64)
    assert np.abs(got - ref).max() <= 1e-5 * np.abs(ref).max(), np.abs(got - ref).max() / np.abs(ref).max()


def test_storage_exact_update_matches_reference_kernel(capi):
    """The storage-exact point update, with cells that take the kept branch
    (small matrix storage, solutions outside [eps, 1 - eps]) and the trial."""
    L = _refk()
    L.refk_storage_exact.argtypes = [dp, dp, dp, dp, dp, dp, ctypes.c_int, dp]
    n = 8
    p = params_for(capi, "c2.params", n=n, pf_y_update_mode=capi.Y_STORAGE_EXACT)
    N = n ** 3
    rng = np.random.default_rng(81)
    phi_new = rng.uniform(0.0, 1.0, N)
    phi_old = np.clip(phi_new + rng.normal(0.0, 0.05, N), 0.0, 1.0)
    phi_new[:20] = 1.0                       # no matrix storage left
    Y_old = rng.uniform(-6.0, 0.5, N)
    divJ = rng.normal(0.0, 2.0, N)
    d = np.array([p.dt, p.v_B, p.Y_clip, p.Y_clip, p.xB_eps, p.gp_h_alpha_eps])
    rY, rx = np.zeros(N), np.zeros(N)
    L.refk_storage_exact(_ptr(divJ), _ptr(phi_new), _ptr(phi_old), _ptr(Y_old), _ptr(rY), _ptr(rx), N, _ptr(d))
    o = _oracle_state(capi, p)
    o.L.pfo_test_storage_exact.argtypes = [ctypes.c_void_p, ctypes.c_double, dp, dp, dp, dp, dp, dp]
    gY, gx = np.zeros(N), np.zeros(N)
    o.L.pfo_test_storage_exact(o.s, p.dt, _ptr(divJ), _ptr(phi_new), _ptr(phi_old), _ptr(Y_old), _ptr(gY), _ptr(gx))
    kept = np.abs(gY - Y_old) < 1e-9
    assert 20 <= kept.sum() < N                  # both branches are exercised
    assert np.abs(gY - rY).max() <= 1e-12 * np.abs(rY).max()
    assert np.abs(gx - rx).max() <= 1e-14


@pytest.mark.parametrize("gp", [0, 1])
def test_flux_matches_reference_kernel(capi, gp):
    """One flux component J = M grad(mu) with the stabilised mobility (D_mix
    over the thermodynamic factor, or the GP-zone phase-weighted form)."""
    L = _refk()
    L.refk_flux.argtypes = [ctypes.c_int, dp, dp, dp, dp, dp, ctypes.c_int, dp]
    n = 8                      # N = 512: the oracle's 1/N scaling is exact
    p = params_for(capi, "c2.params", n=n, model_mode=gp)
    N = n ** 3
    rng = np.random.default_rng(91 + gp)
    g = rng.normal(0.0, 1.0, N)
    phi = rng.uniform(0.0, 1.0, N)
    eta = rng.uniform(0.0, 1.0, N)
    xB = rng.uniform(1e-4, 0.3, N)
    L.refk_set_convex(p.thermo_convex_extrapolation_enabled)
    d = np.array([p.D_alpha, p.D_compound, p.Vm_alpha_0, p.dVm_alpha_dxB, p.Vm_compound, p.temperature_K,
                  p.mu_reference_scale, p.gp_M_GP, p.gp_M_beta])
    ref = np.zeros(N)
    L.refk_flux(gp, _ptr(g), _ptr(phi), _ptr(eta), _ptr(xB), _ptr(ref), N, _ptr(d))
    o = _oracle_state(capi, p)
    o.L.pfo_test_flux.argtypes = [ctypes.c_void_p, dp, dp, dp, dp, dp]
    got = np.zeros(N)
    o.L.pfo_test_flux(o.s, _ptr(g), _ptr(phi), _ptr(eta), _ptr(xB), _ptr(got))
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()


def test_x_split_functions_match_reference_kernels(capi):
    """The x split's storage source (cells below and above the matrix-storage
    floor) and its clamp-and-logit of the new composition (non-finite and
    out-of-range values included)."""
    L = _refk()
    L.refk_xsplit_source.argtypes = [dp, dp, dp, dp, dp, dp, ctypes.c_int, dp]
    L.refk_xsplit_final.argtypes = [dp, dp, dp, ctypes.c_int, dp]
    n = 8                      # N = 512: the oracle's 1/N scaling is exact
    p = params_for(capi, "c2.params", n=n, pf_y_update_mode=capi.Y_X_TRANSPORT_SPLIT)
    N = n ** 3
    rng = np.random.default_rng(101)
    divJ = rng.normal(0.0, 1.0, N)
    phi_new = rng.uniform(0.0, 1.0, N)
    phi_old = rng.uniform(0.0, 1.0, N)
    lap = rng.normal(0.0, 0.1, N)
    xB_old = rng.uniform(1e-3, 0.3, N)
    mDx = p.D_alpha * p.pf_composition_stabilizer_Dalpha_multiplier
    d = np.array([p.dt, p.v_B, mDx, p.pf_matrix_storage_floor])
    ref = np.zeros(N)
    L.refk_xsplit_source(_ptr(divJ), _ptr(phi_new), _ptr(phi_old), _ptr(lap), _ptr(xB_old), _ptr(ref), N, _ptr(d))
    o = _oracle_state(capi, p)
    o.L.pfo_test_xsplit_source.argtypes = [ctypes.c_void_p, ctypes.c_double, dp, dp, dp, dp]
    o.L.pfo_test_xsplit_final.argtypes = [ctypes.c_void_p, ctypes.c_double, dp, dp, dp, dp]
    got = np.zeros(N)
    o.L.pfo_test_xsplit_source(o.s, mDx, _ptr(divJ), _ptr(phi_new), _ptr(lap), _ptr(got))
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()
    x = rng.uniform(-0.05, 1.05, N)
    x[:4] = [np.nan, np.inf, -np.inf, 0.5]
    rx, rY = xB_old.copy(), np.zeros(N)
    L.refk_xsplit_final(_ptr(x), _ptr(rx), _ptr(rY), N, _ptr(np.array([p.xB_eps, p.Y_clip, p.Y_clip])))
    gY, gx = np.zeros(N), np.zeros(N)
    o.L.pfo_test_xsplit_final(o.s, p.dt, _ptr(x), _ptr(xB_old), _ptr(gY), _ptr(gx))
    assert np.abs(gY - rY).max() <= 1e-12 * np.abs(rY).max()
    assert np.abs(gx - rx).max() <= 1e-15


@pytest.mark.parametrize("shape", [(12, 10, 14), (9, 16, 15)])
def test_dealias_matches_reference_kernel(capi, shape):
    """The 2/3 rule with the reference's wave-number wrapping (even and odd
    axis lengths, unequal spacings): the same modes are kept."""
    L = _refk()
    L.refk_dealias.argtypes = [dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                               ctypes.c_double]
    Nx, Ny, Nz = shape
    p = params_for(capi, "c2.params", n=8)
    p.Nx, p.Ny, p.Nz = Nx, Ny, Nz
    p.dx, p.dy, p.dz = 1.0, 0.8, 1.25
    capi.finalize(p)
    Nk = Nx * Ny * (Nz // 2 + 1)
    ones = np.ones(2 * Nk)
    ref = ones.copy()
    L.refk_dealias(_ptr(ref), Nx, Ny, Nz, p.dx, p.dy, p.dz)
    o = _oracle_state(capi, p)
    o.L.pfo_test_dealias.argtypes = [ctypes.c_void_p, dp]
    got = ones.copy()
    o.L.pfo_test_dealias(o.s, _ptr(got))
    assert 0 < (ref == 0).sum() < ref.size
    assert np.array_equal(got, ref)


def test_q_split_functions_match_reference_kernels(capi):
    """The q split's per-cell functions against the reference's kernels: the
    phase storage transfer (feasible and infeasible cells), the explicit
    transport with its bound check (cells inside, below and above [0, 1 - h],
    a non-finite divergence), the bounded reconstruction (out-of-range and
    non-finite q, cells without matrix storage) and the matrix-channel flux."""
    L = _refk()
    L.refk_q_stats_layout.argtypes = [ip, ip]
    L.refk_q_phase.argtypes = [dp, dp, dp, ctypes.c_double, dp, ctypes.c_int]
    L.refk_q_transport.argtypes = [dp, dp, dp, dp, dp, ctypes.c_int, dp, dp]
    L.refk_q_reconstruct.argtypes = [dp, dp, dp, dp, ctypes.c_int, dp, dp]
    L.refk_flux_q.argtypes = [dp, dp, dp, dp, ctypes.c_int, dp]
    n = 8                      # N = 512: the oracle's 1/N scaling is exact
    p = params_for(capi, "c2.params", n=n, pf_y_update_mode=capi.Y_Q_TRANSPORT_SPLIT)
    N = n ** 3
    rng = np.random.default_rng(131)
    i_inf, i_viol = ctypes.c_int(), ctypes.c_int()
    ns = L.refk_q_stats_layout(ctypes.byref(i_inf), ctypes.byref(i_viol))

    def stats():
        st = np.zeros(ns)
        st[7] = 1.0            # PF_Q_MIN_ALPHA starts at 1, as the reference initialises it
        return st

    def h(v):
        v = np.clip(v, 0.0, 1.0)
        return v ** 3 * (6 * v ** 2 - 15 * v + 10)

    o = _oracle_state(capi, p)
    o.L.pfo_test_q_phase.restype = ctypes.c_longlong
    o.L.pfo_test_q_phase.argtypes = [ctypes.c_void_p, dp, dp, dp, dp]
    o.L.pfo_test_q_transport.restype = ctypes.c_longlong
    o.L.pfo_test_q_transport.argtypes = [ctypes.c_void_p, ctypes.c_double, dp, dp, dp, dp, dp, dp, dp]
    o.L.pfo_test_q_reconstruct.argtypes = [ctypes.c_void_p, dp, dp, dp, dp, dp, dp]

    # phase transfer
    phi_old = rng.uniform(-0.05, 1.05, N)
    phi_new = np.clip(phi_old + rng.normal(0.0, 0.2, N), -0.05, 1.05)
    xB = rng.uniform(1e-3, 0.3, N)
    q_in = (1.0 - h(phi_old)) * xB
    rq = q_in.copy()
    st = stats()
    L.refk_q_phase(_ptr(phi_new), _ptr(phi_old), _ptr(rq), p.v_B, _ptr(st), N)
    gq = np.zeros(N)
    bad = o.L.pfo_test_q_phase(o.s, _ptr(phi_new), _ptr(phi_old), _ptr(q_in), _ptr(gq))
    assert 0 < bad < N and bad == int(round(st[i_inf.value]))
    assert np.abs(gq - rq).max() <= 1e-15

    # explicit transport and reconstruction
    phi = rng.uniform(-0.05, 1.05, N)
    phi[:6] = 1.0                      # no matrix storage: x keeps its previous value
    alpha = 1.0 - h(phi)
    q0 = alpha * rng.uniform(1e-3, 0.3, N)
    divJ = rng.normal(0.0, 2.0, N)
    divJ[7] = np.nan
    xB0 = rng.uniform(1e-3, 0.3, N)
    d = np.array([p.dt, p.xB_eps, p.Y_clip, p.Y_clip])
    rq, rx, rY = q0.copy(), xB0.copy(), np.zeros(N)
    st = stats()
    L.refk_q_transport(_ptr(rq), _ptr(divJ), _ptr(phi), _ptr(rx), _ptr(rY), N, _ptr(d), _ptr(st))
    gq, gx, gY = np.zeros(N), np.zeros(N), np.zeros(N)
    viol = o.L.pfo_test_q_transport(o.s, p.dt, _ptr(q0), _ptr(divJ), _ptr(phi), _ptr(xB0), _ptr(gq), _ptr(gx),
                                    _ptr(gY))
    assert 0 < viol < N and viol == int(round(st[i_viol.value]))
    assert np.abs(gq - rq).max() <= 1e-15
    assert np.abs(gx - rx).max() <= 1e-15
    assert np.abs(gY - rY).max() <= 1e-12 * np.abs(rY).max()

    qr = q0 + rng.normal(0.0, 0.05, N)
    qr[:3] = [np.nan, -1.0, 2.0]
    rq, rx, rY = qr.copy(), xB0.copy(), np.zeros(N)
    L.refk_q_reconstruct(_ptr(rq), _ptr(phi), _ptr(rx), _ptr(rY), N, _ptr(d[1:]), _ptr(stats()))
    o.L.pfo_test_q_reconstruct(o.s, _ptr(qr), _ptr(phi), _ptr(xB0), _ptr(gq), _ptr(gx), _ptr(gY))
    assert np.abs(gq - rq).max() <= 1e-15
    assert np.abs(gx - rx).max() <= 1e-15
    assert np.abs(gY - rY).max() <= 1e-12 * np.abs(rY).max()

    # the matrix-channel flux
    g = rng.normal(0.0, 1.0, N)
    L.refk_set_convex(p.thermo_convex_extrapolation_enabled)
    dfl = np.array([p.D_alpha, p.D_compound, p.Vm_alpha_0, p.dVm_alpha_dxB, p.Vm_compound, p.temperature_K,
                    p.mu_reference_scale, p.gp_M_GP, p.gp_M_beta])
    ref = np.zeros(N)
    L.refk_flux_q(_ptr(g), _ptr(phi), _ptr(xB0), _ptr(ref), N, _ptr(dfl))
    o.L.pfo_test_flux.argtypes = [ctypes.c_void_p, dp, dp, dp, dp, dp]
    got = np.zeros(N)
    o.L.pfo_test_flux(o.s, _ptr(g), _ptr(phi), _ptr(phi), _ptr(xB0), _ptr(got))
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()


@pytest.mark.parametrize("ctot", [1, 0])
def test_conservative_functions_match_reference_kernels(capi, ctot):
    """The conservative composition modes' per-cell functions against the
    reference's kernels (ctot_conservative_split and
    qalpha_conservative_local_transaction): the storage from (phi, x), the
    context from the storage (matrix and beta cells), the six checkerboard
    face sweeps in both flux strategies (limited faces included), and the
    phase constraint (capped cells and cells that keep phi^n)."""
    L = _refk()
    L.refk_cons_stats_layout.argtypes = [ip, ip, ip, ip]
    L.refk_cons_init.argtypes = [dp, dp, dp, ctypes.c_double, ctypes.c_int, ctypes.c_int]
    L.refk_cons_context.argtypes = [dp, dp, dp, dp, ctypes.c_int, ctypes.c_int, dp, dp]
    L.refk_cons_sweep.argtypes = [dp, dp, dp, dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                  ctypes.c_int, ctypes.c_int, ctypes.c_int, dp, dp]
    L.refk_cons_constrain.argtypes = [dp, dp, dp, dp, dp, ctypes.c_int, ctypes.c_int, dp, dp]
    n = 8
    mode = capi.COMPOSITION_CTOT if ctot else capi.COMPOSITION_QALPHA
    p = params_for(capi, "c2.params", n=n, pf_composition_mode=mode)
    N = n ** 3
    rng = np.random.default_rng(141 + ctot)
    li, lc, lv, lnf = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    ns = L.refk_cons_stats_layout(ctypes.byref(li), ctypes.byref(lc), ctypes.byref(lv), ctypes.byref(lnf))
    o = _oracle_state(capi, p)
    o.L.pfo_test_cons_init.argtypes = [ctypes.c_void_p, dp, dp, dp]
    o.L.pfo_test_cons_context.argtypes = [ctypes.c_void_p, dp, dp, dp, dp]
    o.L.pfo_test_cons_sweep.restype = ctypes.c_longlong
    o.L.pfo_test_cons_sweep.argtypes = [ctypes.c_void_p, dp, dp, dp, dp, ctypes.c_int, ctypes.c_int, ctypes.c_double]
    o.L.pfo_test_cons_constrain.restype = ctypes.c_longlong
    o.L.pfo_test_cons_constrain.argtypes = [ctypes.c_void_p, dp, dp, dp, dp, dp, ctypes.POINTER(ctypes.c_longlong)]

    phi = rng.uniform(-0.05, 1.05, N)
    phi[:5] = 1.0                              # beta cells: the equilibrium context
    xB = rng.uniform(1e-3, 0.3, N)
    rs, gs = np.zeros(N), np.zeros(N)
    L.refk_cons_init(_ptr(phi), _ptr(xB), _ptr(rs), p.v_B, ctot, N)
    o.L.pfo_test_cons_init(o.s, _ptr(phi), _ptr(xB), _ptr(gs))
    assert np.abs(gs - rs).max() <= 1e-15

    dctx = np.array([p.temperature_K, p.v_B, p.pf_conservative_beta_support_eps, p.xB_eps, p.Y_clip])
    rx, rY, gx, gY = np.zeros(N), np.zeros(N), np.zeros(N), np.zeros(N)
    L.refk_cons_context(_ptr(rs), _ptr(phi), _ptr(rx), _ptr(rY), ctot, N, _ptr(dctx), _ptr(np.zeros(ns)))
    o.L.pfo_test_cons_context(o.s, _ptr(rs), _ptr(phi), _ptr(gx), _ptr(gY))
    assert np.abs(gx - rx).max() <= 1e-15
    assert np.abs(gY - rY).max() <= 1e-12 * np.abs(rY).max()

    mu = rng.normal(0.0, 2.0, N)
    L.refk_set_convex(p.thermo_convex_extrapolation_enabled)
    import oracle_py
    dt = 5.0 * p.dt                            # large enough that some faces hit the storage bounds
    for be in (0, 1):
        rsw, gsw = rs.copy(), rs.copy()
        st = np.zeros(ns)
        ob = oracle_py.Oracle(params_for(capi, "c2.params", n=n, pf_composition_mode=mode, dt=dt,
                                         pf_conservative_flux_strategy=be), threads=1)
        ob.L.pfo_test_cons_sweep.restype = ctypes.c_longlong
        ob.L.pfo_test_cons_sweep.argtypes = o.L.pfo_test_cons_sweep.argtypes
        glim = 0
        for axis, sp in ((0, p.dx), (1, p.dy), (2, p.dz)):
            for par in (0, 1):
                d = np.array([sp, dt, p.D_alpha, p.Vm_alpha_0, p.dVm_alpha_dxB, p.Vm_compound, p.temperature_K,
                              p.mu_reference_scale, p.v_B, p.pf_conservative_bound_tol])
                L.refk_cons_sweep(_ptr(rsw), _ptr(mu), _ptr(phi), _ptr(rx), n, n, n, axis, par, ctot, be, _ptr(d),
                                  _ptr(st))
                glim += ob.L.pfo_test_cons_sweep(ob.s, _ptr(gsw), _ptr(mu), _ptr(phi), _ptr(rx), axis, par, sp)
        assert glim == int(round(st[li.value])) and (be == 1 or glim > 0)
        assert np.abs(gsw - rsw).max() <= 1e-15
        # the sweeps move storage between cells: its sum is unchanged
        assert abs(rsw.sum() - rs.sum()) <= 1e-12 * abs(rs.sum())

    # the phase constraint
    phi_old = np.clip(phi, 0.0, 1.0)
    phi_new = np.clip(phi_old + rng.normal(0.0, 0.3, N), -0.05, 1.05)
    dcon = np.array([p.temperature_K, p.v_B, p.pf_conservative_beta_support_eps, p.xB_eps, p.Y_clip,
                     p.pf_conservative_bound_tol])
    rphi, rst, rx2, rY2 = phi_new.copy(), rsw.copy(), np.zeros(N), np.zeros(N)
    st = np.zeros(ns)
    L.refk_cons_constrain(_ptr(rphi), _ptr(phi_old), _ptr(rst), _ptr(rx2), _ptr(rY2), ctot, N, _ptr(dcon), _ptr(st))
    gphi, gst, gx2, gY2 = phi_new.copy(), rsw.copy(), np.zeros(N), np.zeros(N)
    capped = ctypes.c_longlong()
    bad = o.L.pfo_test_cons_constrain(o.s, _ptr(gphi), _ptr(phi_old), _ptr(gst), _ptr(gx2), _ptr(gY2),
                                      ctypes.byref(capped))
    assert capped.value == int(round(st[lc.value])) and capped.value > 0
    assert bad == int(round(st[lv.value] + st[lnf.value]))
    assert np.abs(gphi - rphi).max() <= 1e-15
    assert np.abs(gst - rst).max() <= 1e-15
    assert np.abs(gx2 - rx2).max() <= 1e-15
    assert np.abs(gY2 - rY2).max() <= 1e-12 * np.abs(rY2).max()


@pytest.mark.parametrize("mode", ["old_rhs", "conservative_y_rhs"])
def test_gp_coupled_y_rhs_matches_reference_kernel(capi, mode):
    """The GP storage-coupled Y right-hand side (GP and beta storage source,
    the gamma term with h_alpha floored at gp_h_alpha_eps in old_rhs, not in
    conservative_y_rhs), both time levels of the gamma term, and the <DY>
    terms h_alpha D_alpha x (1 - x)."""
    L = _refk()
    L.refk_gp_y_rhs.argtypes = [ctypes.c_int, dp, dp, dp, dp, dp, dp, dp, dp, dp, ctypes.c_int, dp, ip]
    L.refk_gp_dy_terms.argtypes = [dp, dp, dp, dp, ctypes.c_double, ctypes.c_int]
    n = 8
    N = n ** 3
    rng = np.random.default_rng(151)
    cons = mode == "conservative_y_rhs"
    for prev in (0, 1):
        p = params_for(capi, "c2.params", n=n, model_mode=1, gp_barrier_only_mode=0,
                       gp_y_update_mode=capi.GP_Y_CONSERVATIVE_RHS if cons else capi.GP_Y_OLD_RHS,
                       enable_Y_rhs_previous_time_level=prev)
        phi = rng.uniform(-1e-6, 1.0, N)
        phi_old = np.clip(phi + rng.normal(0.0, 0.05, N), 0.0, 1.0)
        eta = rng.uniform(0.0, 1.0, N)
        eta[:40] = 1.0                 # no matrix left: the h_alpha floor acts
        eta_old = np.clip(eta + rng.normal(0.0, 0.05, N), 0.0, 1.0)
        Y = rng.uniform(-25.0, 5.0, N)  # beyond the clip at 20 of the source
        lap = rng.normal(0.0, 3.0, N)
        divJ = rng.normal(0.0, 2.0, N)
        dYdt = rng.normal(0.0, 5.0, N)
        mdy = 0.37
        ref = np.zeros(N)
        d = np.array([p.dt, p.gp_xB_fixed, mdy, p.gp_h_alpha_eps])
        iv = (ctypes.c_int * 2)(prev, p.disable_Y_rhs_gamma_term)
        L.refk_gp_y_rhs(int(cons), _ptr(divJ), _ptr(phi), _ptr(phi_old), _ptr(eta), _ptr(eta_old), _ptr(lap),
                        _ptr(Y), _ptr(dYdt), _ptr(ref), N, _ptr(d), iv)
        o = _oracle_state(capi, p)
        o.L.pfo_test_gp_y_rhs.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_double] + [dp] * 9
        got = np.zeros(N)
        o.L.pfo_test_gp_y_rhs(o.s, p.dt, mdy, _ptr(divJ), _ptr(phi), _ptr(phi_old), _ptr(eta), _ptr(eta_old),
                              _ptr(lap), _ptr(Y), _ptr(dYdt), _ptr(got))
        assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max(), (mode, prev)
        # <DY>: the per-cell terms of the reference's reduction, summed
        terms = np.zeros(N)
        L.refk_gp_dy_terms(_ptr(Y), _ptr(phi), _ptr(eta), _ptr(terms), p.D_alpha, N)
        o.L.pfo_test_gp_sum_dy.restype = ctypes.c_double
        o.L.pfo_test_gp_sum_dy.argtypes = [ctypes.c_void_p, dp, dp, dp]
        s = o.L.pfo_test_gp_sum_dy(o.s, _ptr(phi), _ptr(eta), _ptr(Y))
        assert abs(s - terms.sum()) <= 1e-13 * abs(terms.sum())


@pytest.mark.parametrize("mode", ["storage_exact", "picard_storage"])
def test_gp_storage_update_matches_reference_kernel(capi, mode):
    """The GP storage point updates of Y: storage_exact (cells without matrix,
    non-finite and out-of-range solutions, the clip) and three Picard sweeps
    of picard_storage from the guess Y^n."""
    L = _refk()
    L.refk_gp_storage.argtypes = [ctypes.c_int, ctypes.c_int, dp, dp, dp, dp, dp, dp, dp, dp, ctypes.c_int, dp]
    n = 8
    N = n ** 3
    pic = mode == "picard_storage"
    p = params_for(capi, "c2.params", n=n, model_mode=1, gp_barrier_only_mode=0,
                   gp_y_update_mode=capi.GP_Y_PICARD_STORAGE if pic else capi.GP_Y_STORAGE_EXACT)
    rng = np.random.default_rng(161 + pic)
    phi_new = rng.uniform(0.0, 1.0, N)
    phi_old = np.clip(phi_new + rng.normal(0.0, 0.05, N), 0.0, 1.0)
    eta_new = rng.uniform(0.0, 1.0, N)
    eta_old = np.clip(eta_new + rng.normal(0.0, 0.05, N), 0.0, 1.0)
    phi_new[:20] = 1.0                      # no matrix storage left
    Y_old = rng.uniform(-6.0, 0.5, N)
    divJ = rng.normal(0.0, 2.0, N)
    divJ[20] = np.inf                        # non-finite target: Y^n kept
    d = np.array([p.dt, p.gp_xB_fixed, p.Y_clip, p.Y_clip, p.xB_eps, p.gp_h_alpha_eps])
    rY, rx = Y_old.copy(), np.zeros(N)
    L.refk_gp_storage(int(pic), p.gp_y_picard_iters, _ptr(divJ), _ptr(phi_new), _ptr(phi_old), _ptr(eta_new),
                      _ptr(eta_old), _ptr(Y_old), _ptr(rY), _ptr(rx), N, _ptr(d))
    o = _oracle_state(capi, p)
    o.L.pfo_test_gp_storage.argtypes = [ctypes.c_void_p, ctypes.c_double] + [dp] * 9
    gY, gx = np.zeros(N), np.zeros(N)
    o.L.pfo_test_gp_storage(o.s, p.dt, _ptr(divJ), _ptr(phi_new), _ptr(phi_old), _ptr(eta_new), _ptr(eta_old),
                            _ptr(Y_old), _ptr(Y_old), _ptr(gY), _ptr(gx))
    fin = np.isfinite(rY)
    assert fin.all() and np.isfinite(gY).all()
    assert np.abs(gY - rY).max() <= 1e-12 * np.abs(rY).max(), mode
    assert np.abs(gx - rx).max() <= 1e-14
    assert (np.abs(gY - Y_old) < 1e-12).sum() >= 1 and (np.abs(gY - Y_old) > 1e-6).sum() > N // 2


def test_gp_eta_feasibility_matches_reference_kernel(capi):
    """The eta feasibility pass: eta clamped to [0, 1] without the limiter;
    with local_clip the GP fraction lowered (bisection on h_GP, eta by
    inverting h) where the storage target admits no matrix composition in
    [xB_eps, 1 - xB_eps]; the limited-cell count."""
    L = _refk()
    L.refk_gp_eta_feasibility.restype = ctypes.c_double
    L.refk_gp_eta_feasibility.argtypes = [dp, dp, dp, dp, dp, dp, ctypes.c_int, ctypes.c_int, dp]
    n = 8
    N = n ** 3
    p = params_for(capi, "c2.params", n=n, model_mode=1, gp_barrier_only_mode=0,
                   gp_eta_mass_limiter=capi.GP_ETA_LIMITER_LOCAL_CLIP)
    rng = np.random.default_rng(171)
    eta_old = rng.uniform(0.0, 1.0, N)
    eta = np.clip(eta_old + rng.normal(0.0, 0.3, N), -0.1, 1.1)
    phi_old = rng.uniform(0.0, 1.0, N)
    phi_new = np.clip(phi_old + rng.normal(0.0, 0.05, N), 0.0, 1.0)
    xB_old = rng.uniform(1e-4, 0.2, N)
    divJ = rng.normal(0.0, 50.0, N)
    d = np.array([p.dt, p.gp_xB_fixed, p.xB_eps, 1.0 - p.xB_eps, p.gp_h_alpha_eps])
    o = _oracle_state(capi, p)
    o.L.pfo_test_gp_eta_feasibility.restype = ctypes.c_longlong
    o.L.pfo_test_gp_eta_feasibility.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_int] + [dp] * 6
    for lim in (0, 1):
        re, ge = eta.copy(), eta.copy()
        nr = L.refk_gp_eta_feasibility(_ptr(re), _ptr(eta_old), _ptr(phi_new), _ptr(phi_old), _ptr(xB_old),
                                       _ptr(divJ), lim, N, _ptr(d))
        ng = o.L.pfo_test_gp_eta_feasibility(o.s, p.dt, lim, _ptr(ge), _ptr(eta_old), _ptr(phi_new),
                                             _ptr(phi_old), _ptr(xB_old), _ptr(divJ))
        assert int(nr) == ng
        assert np.array_equal(re, ge), lim
        if lim:
            assert ng > 10
        else:
            assert ng == 0 and np.array_equal(ge, np.clip(eta, 0.0, 1.0))


def test_gp_xbtot_matches_reference_kernel(capi):
    """The coupled mass ledger xBtot_gp = h_alpha x + h_GP x_GP + h_beta of
    the diagnostics against the reference's reduction terms."""
    L = _refk()
    L.refk_gp_xbtot_terms.argtypes = [dp, dp, dp, dp, ctypes.c_double, ctypes.c_int]
    n = 8
    N = n ** 3
    p = params_for(capi, "c2.params", n=n, model_mode=1, gp_barrier_only_mode=0)
    rng = np.random.default_rng(181)
    phi = rng.uniform(0.0, 1.0, N)
    eta = rng.uniform(0.0, 1.0, N)
    xB = rng.uniform(1e-3, 0.3, N)
    terms = np.zeros(N)
    L.refk_gp_xbtot_terms(_ptr(phi), _ptr(eta), _ptr(xB), _ptr(terms), p.gp_xB_fixed, N)
    o = _oracle_state(capi, p)
    o.load(phi, xB, eta)
    dg = o.diagnostics(capi.Diag)
    # the oracle's xB is the clipped sigmoid of the loaded logit: xB to rounding
    assert abs(dg.mass_xBtot - terms.sum()) <= 1e-12 * terms.sum()
