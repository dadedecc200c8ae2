"""ctypes wrapper of the CPU oracle (test infrastructure only).

Imported by tests/, __graft_entry__.smoke() and bench.py's CPU baseline; the
product never imports it.  Builds oracle/_build/libpforacle.so on first use.
"""
from __future__ import annotations

import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import build_oracle  # noqa: E402

_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        _LIB = ctypes.CDLL(build_oracle.build_oracle())
        d, vp, i = ctypes.c_double, ctypes.c_void_p, ctypes.c_int
        _LIB.pfo_create.restype = vp
        _LIB.pfo_create.argtypes = [vp]
        _LIB.pfo_destroy.argtypes = [vp]
        _LIB.pfo_load_fields.argtypes = [vp, vp, vp, vp, vp]
        _LIB.pfo_step.argtypes = [vp, i, vp]
        _LIB.pfo_minimize.argtypes = [vp, i, i, vp]
        _LIB.pfo_read_fields.argtypes = [vp, vp, vp, vp, vp, vp]
        _LIB.pfo_read_elastic.argtypes = [vp, vp, vp]
        _LIB.pfo_read_displacement_k.argtypes = [vp, vp]
        _LIB.pfo_diagnostics.argtypes = [vp, vp]
        _LIB.pfo_set_threads.argtypes = [i]
        _LIB.pfo_set_threads.restype = i
        _LIB.pfo_params_finalize.argtypes = [vp]
        _LIB.pfo_fft3d_r2c.argtypes = [i, i, i, vp, vp]
        _LIB.pfo_fft3d_c2r.argtypes = [i, i, i, vp, vp]
        _LIB.pfo_fft1d.argtypes = [i, i, vp, vp]
        for name, k in [("pfo_h", 1), ("pfo_hp", 1), ("pfo_gp", 1), ("pfo_xB_eq", 1),
                        ("pfo_sigmoid", 3), ("pfo_logit", 3), ("pfo_meff", 2)]:
            f = getattr(_LIB, name)
            f.restype = d
            f.argtypes = [d] * k
        for name in ("pfo_mu_A", "pfo_mu_B"):
            f = getattr(_LIB, name)
            f.restype = d
            f.argtypes = [d, d, d, i]
        _LIB.pfo_gamma.restype = d
        _LIB.pfo_gamma.argtypes = [d] * 7 + [i]
    return _LIB


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


class Oracle:
    """One oracle state.  ``params`` is a cuda_sto_pf_gb300.capi.Params."""

    def __init__(self, params, threads: int = 0):
        self.L = lib()
        if threads:
            self.L.pfo_set_threads(threads)
        self.s = self.L.pfo_create(ctypes.byref(params))
        self.shape = (params.Nx, params.Ny, params.Nz)
        self.Nk = params.Nx * params.Ny * (params.Nz // 2 + 1)

    def __del__(self):
        if getattr(self, "s", None):
            self.L.pfo_destroy(self.s)
            self.s = None

    def load(self, phi, xB, eta=None, dYdt=None):
        a = [None if x is None else np.ascontiguousarray(x, dtype=np.float64) for x in (phi, xB, eta, dYdt)]
        self.L.pfo_load_fields(self.s, *[_p(x) for x in a])

    def step(self, n=1, stats=None):
        rc = self.L.pfo_step(self.s, n, None if stats is None else ctypes.byref(stats))
        return rc

    def minimize(self, n=1, stats=None, stop_on_convergence=False):
        return self.L.pfo_minimize(self.s, n, 1 if stop_on_convergence else 0,
                                   None if stats is None else ctypes.byref(stats))

    def fields(self):
        out = {k: np.empty(self.shape) for k in ("phi", "xB", "Y", "eta", "dYdt")}
        self.L.pfo_read_fields(self.s, *[_p(out[k]) for k in ("phi", "xB", "Y", "eta", "dYdt")])
        return out

    def elastic(self):
        sig = np.empty((6,) + self.shape)
        eps = np.empty((6,) + self.shape)
        self.L.pfo_read_elastic(self.s, _p(sig), _p(eps))
        return {"sigma": sig, "strain": eps}

    def displacement_k(self):
        u = np.empty((3, self.Nk, 2))
        self.L.pfo_read_displacement_k(self.s, _p(u))
        return u[..., 0] + 1j * u[..., 1]

    def diagnostics(self, diag_cls):
        d = diag_cls()
        self.L.pfo_diagnostics(self.s, ctypes.byref(d))
        return d


def fft_r2c(x: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float64)
    nx, ny, nz = x.shape
    out = np.empty((nx, ny, nz // 2 + 1), dtype=np.complex128)
    lib().pfo_fft3d_r2c(nx, ny, nz, _p(x), _p(out))
    return out


def fft_c2r(k: np.ndarray, nz: int) -> np.ndarray:
    k = np.ascontiguousarray(k, dtype=np.complex128)
    nx, ny, _ = k.shape
    out = np.empty((nx, ny, nz))
    lib().pfo_fft3d_c2r(nx, ny, nz, _p(k), _p(out))
    return out
