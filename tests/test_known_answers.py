"""Independent known answers (no reference output involved).

The reference ships no golden fields, so besides oracle parity the time step
is pinned to closed-form results that hold exactly on the grid:

* Allen-Cahn single mode.  With W = 0, uniform xB and equal molar volumes
  (c2.params: Vm_alpha_0 = Vm_compound = 1, dVm = 0) the explicit phi drive
  is h'(phi) * dmu with dmu uniform.  For phi = 1/2 + a cos(k x),
  h'(phi) = 30 (1/4 - d^2)^2 with d = a cos(k x) holds only even powers of d,
  so the drive has no Fourier component at k, and one semi-implicit step
  (cuda_kernels.cu:821-843) scales that mode by exactly 1 / (1 + L dt kappa k^2).

* Elastic laminate.  Eigenstrain and stiffness varying along x only: the
  equilibrium sigma_xx is uniform, the other total strains are zero
  (E0 = 0), and <eps_xx> = 0.  With C(x) = C0 + h(phi) dC this gives
      eps_xx = e_xx + (S0 + C12(x) (e_yy + e_zz)) / C11(x),
      S0 = -(<e_xx> + <C12 (e_yy + e_zz) / C11>) / <1 / C11>,
  which the fixed-point elastic iteration (main_cuda.cu:28760-29160) must
  reach.  The profile is band-limited well inside the 2/3 mask, so the
  dealiasing of the spectral solve does not alter the answer.
"""
import os
import sys

import numpy as np
import pytest

from conftest import REPO, params_for


def h_of(phi):
    return phi ** 3 * (6 * phi ** 2 - 15 * phi + 10)


def _mode_case(capi, n, precision):
    p = params_for(capi, "c2.params", n, precision=precision, elastic_enabled=0, W=0.0)
    p.Ny = p.Nz = 4
    capi.finalize(p)
    x = np.arange(n)
    m = 2
    phi = np.broadcast_to((0.5 + 0.1 * np.cos(2 * np.pi * m * x / n))[:, None, None], (n, 4, 4)).copy()
    xB = np.full(phi.shape, 0.03)
    k = 2 * np.pi * m / (n * p.dx)
    factor = 1.0 / (1.0 + p.L_phi * p.dt * p.kappa_phi * k * k)
    return p, phi, xB, m, factor


def _mode_amp(phi, m):
    return np.fft.rfft(phi.mean(axis=(1, 2)))[m]


def test_oracle_phi_single_mode_decay(capi, oracle):
    p, phi, xB, m, factor = _mode_case(capi, 32, capi.PREC_FP64)
    o = oracle(p)
    o.load(phi, xB)
    assert o.step(1) == 0
    out = o.fields()["phi"]
    got = _mode_amp(out, m) / _mode_amp(phi, m)
    assert abs(got - factor) < 1e-12, (got, factor)
    # and the field stays independent of y and z
    assert np.ptp(out, axis=(1, 2)).max() < 1e-14


def laminate_params(capi, n, heterogeneous, precision, elastic_precision, tol):
    over = dict(precision=precision, elastic_precision=elastic_precision, elastic_enabled=1,
                elastic_residual_tolerance=tol, elastic_iter_max=80, elastic_fail_on_nonconvergence=0)
    p = params_for(capi, "c2.params" if heterogeneous else "c1.params", n, **over)
    p.Ny = p.Nz = 4
    capi.finalize(p)
    return p


def laminate_answer(p, phi, xB):
    """Closed-form strain and stress of the x-laminate."""
    S, Sp, e00 = np.array(p.S[:]), np.array(p.S_p[:]), np.array(p.eps00[:])
    h = h_of(phi)
    xc = np.clip(xB, 0.0, 1.0)
    e = [(1 - h) * xc * p.eps_iso_over_vB + h * e00[c] for c in range(3)]
    C = lambda i: S[i] + h * Sp[i]          # noqa: E731  Voigt-21 index
    C11, C12, C13, C22, C23, C33 = C(0), C(1), C(2), C(6), C(7), C(11)
    assert np.allclose(C12, C13)
    rhs = C12 * (e[1] + e[2])
    S0 = -(np.mean(e[0]) + np.mean(rhs / C11)) / np.mean(1.0 / C11)
    exx = e[0] + (S0 + rhs) / C11
    el = [exx - e[0], -e[1], -e[2]]
    sig = [C11 * el[0] + C12 * el[1] + C13 * el[2],
           C12 * el[0] + C22 * el[1] + C23 * el[2],
           C13 * el[0] + C23 * el[1] + C33 * el[2]]
    return exx, sig


def _laminate_fields(n):
    x = np.arange(n)
    phi = np.broadcast_to((0.5 + 0.1 * np.cos(2 * np.pi * x / n))[:, None, None], (n, 4, 4)).copy()
    xB = np.full(phi.shape, 0.03)
    return phi, xB


def _check_laminate(el, p, phi, xB, tol):
    exx, sig = laminate_answer(p, phi, xB)
    eps, s = el["strain"], el["sigma"]
    scale = np.abs(exx).max()
    assert np.abs(eps[0] - exx).max() <= tol * scale
    for c in (1, 2, 3, 4, 5):
        assert np.abs(eps[c]).max() <= tol * scale
    sscale = max(np.abs(sig[1]).max(), np.abs(sig[0]).max())
    for c in range(3):
        assert np.abs(s[c] - sig[c]).max() <= tol * sscale, c
    for c in (3, 4, 5):
        assert np.abs(s[c]).max() <= tol * sscale


@pytest.mark.parametrize("heterogeneous", [False, True])
def test_oracle_elastic_laminate(capi, oracle, heterogeneous):
    n = 32
    p = laminate_params(capi, n, heterogeneous, capi.PREC_FP64, capi.PREC_FP64, 1e-14)
    phi, xB = _laminate_fields(n)
    o = oracle(p)
    o.load(phi, xB)
    st = capi.StepStats()
    assert o.step(1, st) == 0
    assert st.elastic_converged == 1
    # the heterogeneous answer is reached to the fixed point's stopping residual
    _check_laminate(o.elastic(), p, phi, xB, 1e-10 if heterogeneous else 1e-12)


# ----------------------------------------------------------------------------
# the same answers from the CUDA path (through the C ABI)
# ----------------------------------------------------------------------------
@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [(0, 1e-12), (1, 2e-6)])
def test_gpu_phi_single_mode_decay(capi, precision, tol):
    from cuda_sto_pf_gb300.solver import Solver
    p, phi, xB, m, factor = _mode_case(capi, 32, precision)
    with Solver(p) as s:
        s.load(phi, xB)
        s.step(1)
        out = s.fields()["phi"]
    got = _mode_amp(out, m) / _mode_amp(phi, m)
    assert abs(got - factor) < tol, (got, factor)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("heterogeneous", [False, True])
def test_gpu_elastic_laminate(capi, heterogeneous, precision):
    from cuda_sto_pf_gb300.solver import Solver
    n = 32
    p = laminate_params(capi, n, heterogeneous, precision, capi.PREC_FP32, 1e-6)
    phi, xB = _laminate_fields(n)
    with Solver(p) as s:
        s.load(phi, xB)
        st = s.step(1)
        assert st.elastic_converged == 1
        el = s.elastic()
    _check_laminate(el, p, phi, xB, 2e-5)


def test_chebyshev_bounds_match_generalised_eigenvalues(capi):
    """The oracle's spectral bounds of the elastic increment operator are
    [min(0, -mu_max), max(0, -mu_min)] widened by 2%, mu the generalised
    eigenvalues of (dC, C0) in Voigt form."""
    import ctypes
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle_py
    L = oracle_py.lib()
    dp = ctypes.POINTER(ctypes.c_double)
    L.pfo_chebyshev_bounds.restype = ctypes.c_int
    L.pfo_chebyshev_bounds.argtypes = [dp, dp, dp, dp]
    p = params_for(capi, "c2.params", n=16)
    a, b = ctypes.c_double(), ctypes.c_double()
    assert L.pfo_chebyshev_bounds(p.S, p.S_p, ctypes.byref(a), ctypes.byref(b)) == 1
    st = [0, 6, 11, 15, 18, 20]
    V = lambda c, i, j: c[st[min(i, j)] + max(i, j) - min(i, j)]
    C0 = np.array([[V(p.S, i, j) for j in range(6)] for i in range(6)])
    dC = np.array([[V(p.S_p, i, j) for j in range(6)] for i in range(6)])
    mu = np.linalg.eigvals(np.linalg.solve(C0, dC)).real
    lo, hi = min(0.0, -mu.max()), max(0.0, -mu.min())
    w = 0.02 * (hi - lo)
    assert abs(a.value - (lo - w)) < 1e-12 and abs(b.value - (hi + w)) < 1e-12
    # a contrast whose bound reaches 1 is refused
    Sp = np.array(p.S[:]) * -1.2
    arr = (ctypes.c_double * 21)(*Sp)
    assert L.pfo_chebyshev_bounds(p.S, arr, ctypes.byref(a), ctypes.byref(b)) == 0
