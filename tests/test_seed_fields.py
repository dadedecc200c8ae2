"""Seeded initial fields (initialize_fields_cuda, main_cuda.cu:15157-15430):
the device initialiser against its numpy restatement (oracle/init_oracle.py)
for a centred sphere, a tilted ellipsoid with a shifted centre, and several
randomly placed seeds with phi noise and the lever-rule composition."""
import ctypes
import os
import sys

import numpy as np
import pytest

from conftest import REPO, params_for

sys.path.insert(0, os.path.join(REPO, "oracle"))
import init_oracle  # noqa: E402

CASES = {
    "sphere": dict(),
    "tilted_ellipsoid": dict(init_shape_mode=1, init_axis_ratio_rx=1.0, init_axis_ratio_ry=0.7,
                             init_axis_ratio_rz=0.4, init_use_rotation=1, init_tilt_theta_deg=35.0,
                             init_tilt_phi_deg=20.0, init_center_shift_x=3.5, init_center_shift_z=-2.0),
    "seeds_noise_lever": dict(ic_phi_num_seeds=5, ic_phi_seed_radius=4.0, seed=777, init_phi_noise_amp=0.02,
                              ic_23d_xB_out=-1.0, ic_vf_target_phi=0.05),
}


def _params(capi, case, n=32):
    p = params_for(capi, "c2.params", n=n, **CASES[case])
    return p


def test_oracle_sphere_profile(capi):
    p = _params(capi, "sphere", n=24)
    phi, xB = init_oracle.seed_fields(p)
    w = p.ic_phi_iface_w * p.dx
    R = p.ic_phi_seed_radius
    c = 12
    assert abs(phi[c, c, c] - 0.5 * (1 + np.tanh(R / w))) < 1e-14   # centre cell: r_eff = 0
    assert np.allclose(xB[0, 0, 0], max(p.ic_23d_xB_out, p.xB_eps), atol=1e-9)
    # translation by the centre shift moves the field by whole cells
    p2 = _params(capi, "sphere", n=24)
    p2.init_center_shift_x = 3 * p2.dx
    phi2, _ = init_oracle.seed_fields(p2)
    assert np.abs(np.roll(phi, 3, axis=0) - phi2).max() < 1e-12


def test_oracle_noise_is_uniform_and_bounded(capi):
    u = init_oracle._noise_u(200000, 12345)
    assert 0.0 <= u.min() and u.max() <= 1.0
    assert abs(u.mean() - 0.5) < 5e-3 and abs(u.var() - 1 / 12) < 5e-3


@pytest.mark.gpu
@pytest.mark.parametrize("case", list(CASES))
def test_seed_fields_match_oracle(capi, case):
    from cuda_sto_pf_gb300.solver import Solver
    p = _params(capi, case)
    want_phi, want_xB = init_oracle.seed_fields(p)
    N = p.Nx * p.Ny * p.Nz
    phi, xB = np.empty(N), np.empty(N)
    capi.check(capi.load().pfgb_seed_fields(ctypes.byref(p), 0, phi.ctypes.data, xB.ctypes.data), "seed_fields")
    assert np.abs(phi.reshape(want_phi.shape) - want_phi).max() <= 1e-12
    assert np.abs(xB.reshape(want_xB.shape) - want_xB).max() <= 1e-12
    if case == "seeds_noise_lever":
        assert want_phi.max() > 0.9 and np.unique(np.round(want_phi, 3)).size > 100
    # the context initialiser loads the same state
    p.precision = 0
    with Solver(p) as s:
        capi.check(s.lib.pfgb_init_fields(s.ctx), "pfgb_init_fields")
        f = s.fields()
    assert np.abs(f["phi"] - want_phi).max() <= 1e-12
    assert np.abs(f["xB"] - want_xB).max() <= 1e-9
