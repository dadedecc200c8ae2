"""Minimize mode (--mode=minimize --minimize-full-model): the oracle's
iteration against its own invariants, and the CUDA path against the oracle
through the C ABI (main_cuda.cu:29264-29750, 32100-32600)."""
import ctypes

import numpy as np
import pytest

from conftest import params_for, rel_l2


def _case(capi, n=32, precision=0, **over):
    from cuda_sto_pf_gb300 import workloads
    kw = dict(mode=capi.MODE_MINIMIZE, minimize_full_model=1, minimize_dt=0.05, precision=precision)
    kw.update(over)
    p = params_for(capi, "c2.params", n=n, **kw)
    w = workloads.single_sphere(n=n, radius=8.0)
    phi, xB = w["phi"], w["xB"]
    capi.load().pfgb_prepare_raw_fields(ctypes.byref(p), 0.07, phi.ctypes.data, xB.ctypes.data, None, None,
                                        phi.size)
    return p, phi, xB


FIELDS = ("mean_h", "lambda_vol", "F_surf", "F_el", "F_chem_excess", "F_total_excess",
          "rms_res", "rms_dphi", "rms_dY", "vol_err_rel")


def test_oracle_minimize_invariants(capi, oracle):
    p, phi, xB = _case(capi, n=24)
    o = oracle(p, threads=4)
    o.load(phi, xB)
    ms = capi.MinStats()
    out = []
    for _ in range(6):
        assert o.minimize(1, ms) == 0
        out.append((ms.mean_h, ms.V0_target, ms.F_total_excess, ms.rms_res, ms.vol_err_rel))
    # V0 <= 0: the legacy seed-radius target (one sphere of ic_phi_seed_radius)
    R, L = p.ic_phi_seed_radius, 24 * p.dx
    assert abs(out[0][1] - 4.0 / 3.0 * np.pi * R ** 3 / L ** 3) < 1e-12
    # the V0 projection holds <h> on the target after the first iterations
    assert all(v[4] < 1e-4 for v in out[2:])
    # the projected KKT residual decreases along the flow
    assert out[-1][3] < out[1][3]


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [(0, 1e-6), (1, 2e-5)])
def test_minimize_parity(capi, oracle, precision, tol):
    from cuda_sto_pf_gb300.solver import Solver
    p, phi, xB = _case(capi, precision=precision, minimize_V0=0.1)
    o = oracle(p, threads=8)
    o.load(phi, xB)
    mo, mg = capi.MinStats(), capi.MinStats()
    with Solver(p) as s:
        s.load(phi, xB)
        for it in range(6):
            assert o.minimize(1, mo) == 0
            s.minimize(1, mg)
            assert mg.iteration == mo.iteration == it + 1
            for f in FIELDS:
                a, b = getattr(mg, f), getattr(mo, f)
                if f == "vol_err_rel":
                    # |<h> - V0| / V0 is a difference of nearly equal volumes: an
                    # absolute bound at the field precision (FP32 phi: ~1e-7)
                    assert abs(a - b) <= (1e-10 if precision == 0 else 1e-7), (it, f, a, b)
                    continue
                scale = max(abs(b), 1e-6 if f.startswith("rms") else 1e-12)
                assert abs(a - b) <= (50 * tol if f == "rms_res" else tol) * scale, (it, f, a, b)
            assert mg.xB_clamped == mo.xB_clamped
            assert abs(mg.elastic_iterations - mo.elastic_iterations) <= 1
        fg = s.fields()
    fo = o.fields()
    for k in ("phi", "xB", "Y"):
        assert rel_l2(fg[k], fo[k]) <= tol, k


PHI_ONLY_FIELDS = ("mean_h", "lambda_vol", "F_surf", "F_el", "rms_res", "rms_dphi", "vol_err_rel")


def test_oracle_phi_only_minimize(capi, oracle):
    """minimize_full_model = 0 (the reference's default minimize): no
    composition, so the chemical energies and rms_dY are NaN and the
    composition does not move; the volume projection and the KKT residual
    behave as in the full model."""
    p, phi, xB = _case(capi, n=24, minimize_full_model=0, minimize_V0=0.1)
    o = oracle(p, threads=4)
    o.load(phi, xB)
    ms = capi.MinStats()
    res = []
    for _ in range(6):
        assert o.minimize(1, ms) == 0
        assert np.isnan(ms.F_chem_excess) and np.isnan(ms.F_total_excess) and np.isnan(ms.rms_dY)
        assert np.isnan(ms.F_chem_CNT) and ms.condB == 0 and ms.xB_clamped == 0
        res.append((ms.rms_res, ms.vol_err_rel, ms.F_el))
    assert all(v[1] < 1e-4 for v in res[2:])
    assert res[-1][0] < res[1][0]
    assert all(v[2] > 0 for v in res)


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [(0, 1e-6), (1, 2e-5)])
def test_phi_only_minimize_parity(capi, oracle, precision, tol):
    """Phi-only minimize (compute_phi_rhs_minimize_kernel, cuda_kernels.cu:6298-6374;
    the phi-only eigenstrain h(phi) eps00) on the GPU against the oracle,
    iteration by iteration, heterogeneous elasticity, V0 = 0.1."""
    from cuda_sto_pf_gb300.solver import Solver
    p, phi, xB = _case(capi, precision=precision, minimize_full_model=0, minimize_V0=0.1)
    o = oracle(p, threads=8)
    o.load(phi, xB)
    mo, mg = capi.MinStats(), capi.MinStats()
    with Solver(p) as s:
        s.load(phi, xB)
        for it in range(6):
            assert o.minimize(1, mo) == 0
            s.minimize(1, mg)
            assert mg.iteration == mo.iteration == it + 1
            for f in ("F_chem_excess", "F_total_excess", "F_chem_CNT", "F_total_CNT", "rms_dY"):
                assert np.isnan(getattr(mg, f)), f
            for f in PHI_ONLY_FIELDS:
                a, b = getattr(mg, f), getattr(mo, f)
                if f == "vol_err_rel":
                    # the phi-only drive is mostly elastic, so the FP32
                    # elastic rounding (different transform orders on the two
                    # sides) reaches <h> at about 1e-8 relative even with
                    # FP64 fields
                    assert abs(a - b) <= (5e-9 if precision == 0 else 1e-7), (it, f, a, b)
                    continue
                scale = max(abs(b), 1e-6 if f.startswith("rms") else 1e-12)
                assert abs(a - b) <= (50 * tol if f == "rms_res" else tol) * scale, (it, f, a, b)
            assert (mg.condA, mg.condB, mg.xB_clamped) == (mo.condA, mo.condB, 0)
            assert abs(mg.elastic_iterations - mo.elastic_iterations) <= 1
        fg = s.fields()
    fo = o.fields()
    assert rel_l2(fg["phi"], fo["phi"]) <= tol


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [(0, 1e-6), (1, 2e-5)])
def test_gp_zone_minimize_parity(capi, oracle, precision, tol):
    """Full-model minimize in gp_zone (GP elasticity on phi and eta): eta is
    held fixed (it evolves in dynamics only), the phi drive, the flux mu and
    the eigenstrain take their GP forms.  GPU against the oracle, iteration
    by iteration."""
    from cuda_sto_pf_gb300 import workloads
    from cuda_sto_pf_gb300.solver import Solver
    p, phi, xB = _case(capi, precision=precision, minimize_V0=0.1, model_mode=1, gp_elastic_enabled=1,
                       gp_elastic_active_phi=1, gp_elastic_active_eta=1)
    eta = workloads.ellipsoid_field(phi.shape, [np.array([5.0, 5.0, 5.0])], [np.full(3, 3.0)], [np.eye(3)],
                                    p.ic_phi_iface_w)
    o = oracle(p, threads=8)
    o.load(phi, xB, eta)
    mo, mg = capi.MinStats(), capi.MinStats()
    with Solver(p) as s:
        s.load(phi, xB, eta)
        for it in range(5):
            assert o.minimize(1, mo) == 0
            s.minimize(1, mg)
            for f in FIELDS:
                a, b = getattr(mg, f), getattr(mo, f)
                if f == "vol_err_rel":
                    assert abs(a - b) <= (1e-9 if precision == 0 else 1e-7), (it, f, a, b)
                    continue
                scale = max(abs(b), 1e-6 if f.startswith("rms") else 1e-12)
                assert abs(a - b) <= (50 * tol if f == "rms_res" else tol) * scale, (it, f, a, b)
            assert abs(mg.elastic_iterations - mo.elastic_iterations) <= 1
        fg = s.fields()
    fo = o.fields()
    for k in ("phi", "xB", "Y"):
        assert rel_l2(fg[k], fo[k]) <= tol, k
    assert rel_l2(fg["eta"], eta) == 0.0 or rel_l2(fg["eta"], eta) <= 1e-7   # eta unchanged


@pytest.mark.gpu
def test_minimize_stops_on_convergence(capi):
    from cuda_sto_pf_gb300.solver import Solver
    big = 1e30
    p, phi, xB = _case(capi, n=16, precision=1, minimize_convergence_steps=3, minimize_rms_dphi_threshold=big,
                       minimize_rms_dY_threshold=big, minimize_rms_res_threshold=big,
                       minimize_vol_err_rel_threshold=big, minimize_energy_diff_rel_threshold=big)
    with Solver(p) as s:
        s.load(phi, xB)
        st = s.minimize(10, stop_on_convergence=True)
        assert st.converged == 1 and st.converged_iteration == 3 and st.iteration == 3
        # a dynamics call on a minimize context is refused
        with pytest.raises(capi.PfgbError):
            s.step(1)


@pytest.mark.gpu
def test_minimize_on_dynamics_context_is_refused(capi):
    from cuda_sto_pf_gb300.solver import Solver
    p = params_for(capi, "c2.params", n=16)
    from cuda_sto_pf_gb300 import workloads
    w = workloads.single_sphere(n=16, radius=5.0)
    with Solver(p) as s:
        s.load(w["phi"], w["xB"])
        with pytest.raises(capi.PfgbError):
            s.minimize(1)
