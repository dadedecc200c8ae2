"""The extrapolated start of the heterogeneous elastic solve
(elastic_warm_start_extrapolate = 0..5) on the oracle: a size-independent
property of the scheme.  Every order reaches the same fixed point (the
fields agree to the elastic tolerance's effect on them), and the iteration
count does not grow with the order once the history has filled.  CPU only."""
import ctypes

import numpy as np

from conftest import params_for, rel_l2


def _run(capi, oracle, order, n=24, steps=9):
    from cuda_sto_pf_gb300 import workloads
    p = params_for(capi, "c2.params", n=n, elastic_residual_tolerance=1e-8, elastic_fail_on_nonconvergence=0,
                   elastic_chebyshev=1, elastic_warm_start_extrapolate=order)
    rng = np.random.default_rng(41)
    phi = workloads.ellipsoid_field((n, n, n), [np.full(3, n / 2.0)], [np.array([6.0, 5.0, 4.0])],
                                    [workloads.random_rotation(rng)], p.ic_phi_iface_w)
    xB = workloads.composition(phi, rng)
    assert capi.load().pfgb_prepare_raw_fields(ctypes.byref(p), 0.07, phi.ctypes.data, xB.ctypes.data, None,
                                               None, phi.size) == 0
    o = oracle(p, threads=8)
    o.load(phi, xB)
    its = []
    for _ in range(steps):
        st = capi.StepStats()
        assert o.step(1, st) == 0
        assert st.elastic_converged == 1
        its.append(st.elastic_iterations)
    return its, o.fields()


def test_extrapolated_starts_share_the_fixed_point(capi, oracle):
    runs = {m: _run(capi, oracle, m) for m in range(6)}
    base_its, base = runs[0]
    for m in range(1, 6):
        its, f = runs[m]
        # the cold step and the first warm one (one solution in the history)
        # start from the same point whatever the order
        assert its[:2] == base_its[:2], (m, its, base_its)
        for k in ("phi", "xB", "Y"):
            assert rel_l2(f[k], base[k]) <= 1e-8, (m, k, rel_l2(f[k], base[k]))
    tail = {m: sum(runs[m][0][-3:]) for m in range(6)}
    for m in range(1, 6):
        assert tail[m] <= tail[m - 1], tail
    assert tail[5] < tail[1] < tail[0], tail
