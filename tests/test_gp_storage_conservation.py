"""Size-independent properties of the GP storage coupling's point updates
on the oracle (gp_zone, gp_barrier_only_mode = 0).  storage_exact solves
xBtot_gp^{n+1} = xBtot_gp^n + dt div J per cell, and the periodic
divergence sums to zero, so where no cell leaves the composition bounds or
the h_alpha floor the total xBtot_gp is conserved to round-off;
picard_storage's sweeps converge to that balance, so their drift falls with
the sweep count.  A gentle case (phi and eta of amplitude 0.35 and 0.3,
dt = 1e-4) keeps every cell inside the bounds.  CPU only."""
import numpy as np

from conftest import params_for


def _drift(capi, oracle, mode, iters=3, n=24, steps=5):
    from cuda_sto_pf_gb300 import workloads
    p = params_for(capi, "c2.params", n=n, model_mode=1, gp_barrier_only_mode=0, gp_y_update_mode=mode, dt=1e-4,
                   gp_y_picard_iters=iters)
    rng = np.random.default_rng(3)
    phi = 0.35 * workloads.ellipsoid_field((n, n, n), [np.full(3, n / 2.0)], [np.array([6.0, 5.0, 4.0])],
                                           [workloads.random_rotation(rng)], p.ic_phi_iface_w)
    eta = 0.3 * workloads.ellipsoid_field((n, n, n), [np.full(3, 6.0)], [np.full(3, 4.0)], [np.eye(3)],
                                          p.ic_phi_iface_w)
    xB = 0.03 + 1e-3 * rng.standard_normal(phi.shape)
    o = oracle(p, threads=8)
    o.load(phi, xB, eta)
    m0 = o.diagnostics(capi.Diag).mass_xBtot
    worst = 0.0
    for _ in range(steps):
        st = capi.StepStats()
        assert o.step(1, st) == 0
        worst = max(worst, abs(o.diagnostics(capi.Diag).mass_xBtot - m0) / m0)
    f = o.fields()
    assert f["xB"].min() > 0.02 and f["xB"].max() < 0.04   # inside the bounds throughout
    return worst


def test_storage_exact_conserves_xbtot_gp(capi, oracle):
    assert _drift(capi, oracle, capi.GP_Y_STORAGE_EXACT) <= 1e-13


def test_picard_storage_converges_to_the_balance(capi, oracle):
    d = [_drift(capi, oracle, capi.GP_Y_PICARD_STORAGE, iters=k) for k in (3, 10, 30)]
    assert d[0] > d[1] > d[2], d
    assert d[2] <= 1e-13, d
