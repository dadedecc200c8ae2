"""Pin the oracle's restatement of the reference thermodynamics and phase
functions (thermo_utils.h, phase_functions.h) against golden vectors produced
by the reference headers compiled on the host (tests/golden/make_golden.py),
and, where the reference tree is present, against the compiled reference
directly on random inputs."""
import ctypes
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, REPO


@pytest.fixture(scope="module")
def golden():
    with open(os.path.join(GOLDEN, "thermo_golden.json")) as f:
        return json.load(f)


def _close(a, b, ulps=2):
    if a == b:
        return True
    return abs(a - b) <= ulps * np.spacing(max(abs(a), abs(b)))


def test_phase_functions(oracle, golden):
    import oracle_py
    L = oracle_py.lib()
    for p, h, hp, gp in golden["phase"]:
        assert _close(L.pfo_h(p), h) and _close(L.pfo_hp(p), hp) and _close(L.pfo_gp(p), gp)


def test_chemical_potentials(oracle, golden):
    import oracle_py
    L = oracle_py.lib()
    for convex, x, T, s, muA, muB in golden["mu"]:
        assert _close(L.pfo_mu_A(x, T, s, int(convex)), muA), (convex, x, T, s)
        assert _close(L.pfo_mu_B(x, T, s, int(convex)), muB), (convex, x, T, s)


def test_thermodynamic_factor(oracle, golden):
    import oracle_py
    L = oracle_py.lib()
    for convex, x, h, vm0, dvm, vmc, T, s, g in golden["gamma"]:
        got = L.pfo_gamma(x, h, vm0, dvm, vmc, T, s, int(convex))
        # central difference of rounded potentials: allow a few ulps of mu / dx
        assert got == pytest.approx(g, rel=1e-12, abs=1e-12 * abs(g) + 1e-14), (convex, x, h, T, s)


def test_solubility_sigmoid_logit(oracle, golden):
    import oracle_py
    L = oracle_py.lib()
    for T, x in golden["xB_eq"]:
        assert _close(L.pfo_xB_eq(T), x)
    for Y, Yc, eps, x in golden["sigmoid"]:
        assert _close(L.pfo_sigmoid(Y, Yc, eps), x)
    for x, eps, Yc, Y in golden["logit"]:
        assert _close(L.pfo_logit(x, eps, Yc), Y)


REF_LIB = os.path.join(REPO, "oracle", "_ref", "libpfref.so")


@pytest.mark.skipif(not os.path.exists(REF_LIB), reason="reference pin library not built here")
def test_against_compiled_reference_random(oracle):
    import oracle_py
    L = oracle_py.lib()
    R = ctypes.CDLL(REF_LIB)
    d = ctypes.c_double
    R.ref_mu_A.restype = R.ref_mu_B.restype = d
    R.ref_mu_A.argtypes = R.ref_mu_B.argtypes = [d] * 3
    R.ref_gamma.restype = d
    R.ref_gamma.argtypes = [d] * 7
    R.ref_set_convex.argtypes = [ctypes.c_int]
    rng = np.random.default_rng(7)
    for convex in (0, 1):
        R.ref_set_convex(convex)
        for _ in range(3000):
            x = float(10 ** rng.uniform(-8, -0.01))
            T = float(rng.uniform(500, 1400))
            s = float(rng.uniform(1e3, 3e4))
            h = float(rng.uniform(0, 1))
            assert _close(L.pfo_mu_A(x, T, s, convex), R.ref_mu_A(x, T, s))
            assert _close(L.pfo_mu_B(x, T, s, convex), R.ref_mu_B(x, T, s))
            g = R.ref_gamma(x, h, 1.0, 0.0, 1.0, T, s)
            assert L.pfo_gamma(x, h, 1.0, 0.0, 1.0, T, s, convex) == pytest.approx(g, rel=1e-12)
    R.ref_set_convex(0)
