"""Batched minimize sweep (pfgb_batch_minimize): cases of different grids
and eigenstrain directions share the device; each case's result equals the
same case run alone through pfgb_minimize."""
import ctypes

import numpy as np
import pytest

from conftest import params_for


def test_sweep_cases_follow_the_config():
    from cuda_sto_pf_gb300 import workloads
    cs = workloads.sweep_cases()
    assert len(cs) == 48
    assert sorted({c["n"] for c in cs}) == [64, 80, 96, 112, 128, 144, 160]
    assert {c["ca"] for c in cs} <= {1.0, 0.6, 0.3}
    assert all(10.0 <= c["radius"] <= 40.0 and c["radius"] < c["n"] / 2 - 5 for c in cs)
    for c in cs:
        e = c["eps00"]
        # a rotation keeps the trace and the eigenvalues of diag(0.046, -0.022, -0.017)
        E = np.array([[e[0], e[5], e[4]], [e[5], e[1], e[3]], [e[4], e[3], e[2]]])
        assert abs(np.trace(E) - 0.007) < 1e-12
        assert np.allclose(np.sort(np.linalg.eigvalsh(E)), [-0.022, -0.017, 0.046])


def _case_params(capi, case, iters):
    p = params_for(capi, "c2.params", n=case["n"], mode=capi.MODE_MINIMIZE, minimize_full_model=1,
                   minimize_dt=0.05, minimize_V0=0.1, precision=1, eps00=case["eps00"])
    return p


@pytest.mark.gpu
def test_batch_minimize_equals_single_runs(capi):
    from cuda_sto_pf_gb300 import workloads
    from cuda_sto_pf_gb300.solver import Solver
    lib = capi.load()
    specs = [dict(c, n=n, radius=5.0) for c, n in zip(workloads.sweep_cases(count=4), (16, 64, 40, 96))]
    iters = 4
    arr = (capi.Case * len(specs))()
    keep = []
    for i, c in enumerate(specs):
        f = workloads.spheroid_fields(c)
        p = _case_params(capi, c, iters)
        lib.pfgb_prepare_raw_fields(ctypes.byref(p), 0.07, f["phi"].ctypes.data, f["xB"].ctypes.data, None, None,
                                    f["phi"].size)
        out = np.empty_like(f["phi"])
        keep.append((p, f, out))
        arr[i].params = p
        arr[i].phi = f["phi"].ctypes.data
        arr[i].xB = f["xB"].ctypes.data
        arr[i].phi_out = out.ctypes.data
        arr[i].max_iter = iters
    assert lib.pfgb_batch_minimize(arr, len(specs), 0, 3) == 0
    for i, (p, f, out) in enumerate(keep):
        assert arr[i].status == 0 and arr[i].stats.iteration == iters
        with Solver(p) as s:
            s.load(f["phi"], f["xB"])
            st = s.minimize(iters)
            ref = s.fields()["phi"]
        assert np.array_equal(out, ref), i
        assert st.F_total_excess == arr[i].stats.F_total_excess
